// Request scheduler for serving many independent Poisson solves on one GPU.
//
// Operators (nrsg_elliptic handles) stay resident: mesh, geometric factors
// and multigrid hierarchy are built once.  A request names a handle, its
// device right-hand side and solution buffers and a tolerance.  Requests
// wait in arrival order; step() admits the head of the queue whenever its
// handle is idle and the device footprint of the handles with requests in
// flight stays within the budget (a request always starts when nothing is in
// flight), then advances every request in flight by at most one Krylov
// iteration with the non-blocking resumable solve (nrsg_elliptic_solve_begin /
// _advance): each handle runs on its own stream, so the iterations of all
// requests in flight overlap on the device.  A request that waits for a busy
// handle does not block the requests behind it.  Finished requests are
// collected with poll().  The reference has no serving loop; its solve is
// the blocking ellipticSolve (src/solvers/elliptic/ellipticSolve.cpp:32-190).

#include "nrsg_internal.hpp"

#include <deque>
#include <mutex>
#include <unordered_set>
#include <vector>

struct nrsg_elliptic; // C-ABI handle (elliptic.cu)

namespace {
struct Request {
  long long id;
  nrsg_elliptic *el;
  double *r, *x;
  double tol;
  int relative, maxIter;
  long long bytes;
};
} // namespace

struct nrsg_server {
  std::mutex m;
  long long budget = 0, inflightBytes = 0, nextId = 1;
  std::deque<Request> queue;
  std::vector<Request> active;
  std::unordered_set<nrsg_elliptic *> busy;
  std::deque<std::pair<long long, nrsg_solve_info>> done;
  std::deque<int> doneCode;
};

extern "C" {

int nrsg_server_create(long long hbm_budget_bytes, nrsg_server **out)
{
  if (!out || hbm_budget_bytes < 0) return NRSG_ERR_INVALID;
  try {
    auto *s = new nrsg_server();
    s->budget = hbm_budget_bytes;
    *out = s;
    return NRSG_OK;
  } catch (const std::bad_alloc &) {
    nrsg::set_last_error("host allocation failed");
    return NRSG_ERR_OOM;
  }
}

int nrsg_server_destroy(nrsg_server *s)
{
  if (!s) return NRSG_ERR_INVALID;
  if (!s->active.empty()) {
    nrsg::set_last_error("server: requests are still in flight");
    return NRSG_ERR_INVALID;
  }
  delete s;
  return NRSG_OK;
}

int nrsg_server_submit(nrsg_server *s, nrsg_elliptic *el, double *d_r, double *d_x, double tol, int relative,
                       int maxIterations, long long footprint_bytes, long long *request_id)
{
  if (!s || !el || !d_r || !d_x || !request_id || footprint_bytes < 0) return NRSG_ERR_INVALID;
  std::lock_guard<std::mutex> lock(s->m);
  Request q{s->nextId++, el, d_r, d_x, tol, relative, maxIterations, footprint_bytes};
  s->queue.push_back(q);
  *request_id = q.id;
  return NRSG_OK;
}

int nrsg_server_step(nrsg_server *s, int *in_flight, int *queued)
{
  if (!s) return NRSG_ERR_INVALID;
  std::lock_guard<std::mutex> lock(s->m);
  // admission: arrival order, skipping requests whose handle is busy
  for (auto it = s->queue.begin(); it != s->queue.end();) {
    const bool fits = s->active.empty() || s->inflightBytes + it->bytes <= s->budget;
    if (!fits) break; // the budget is full: later requests wait too (arrival order)
    if (s->busy.count(it->el)) {
      ++it;
      continue;
    }
    Request q = *it;
    int code = nrsg_elliptic_set_tolerance(q.el, q.tol, q.relative, q.maxIter);
    if (code == NRSG_OK) code = nrsg_elliptic_solve_begin(q.el, q.r, q.x);
    it = s->queue.erase(it);
    if (code != NRSG_OK) { // did not start: reported as finished with its error
      nrsg_solve_info info{};
      info.status = code;
      s->done.push_back({q.id, info});
      s->doneCode.push_back(code);
      continue;
    }
    s->busy.insert(q.el);
    s->inflightBytes += q.bytes;
    s->active.push_back(q);
  }
  // one non-blocking advance of every request in flight
  for (size_t k = 0; k < s->active.size();) {
    Request &q = s->active[k];
    int fin = 0;
    nrsg_solve_info info{};
    const int code = nrsg_elliptic_solve_advance(q.el, &fin, &info);
    if (fin) {
      if (info.status == NRSG_OK && code != NRSG_OK) info.status = code;
      s->done.push_back({q.id, info});
      s->doneCode.push_back(code);
      s->busy.erase(q.el);
      s->inflightBytes -= q.bytes;
      s->active.erase(s->active.begin() + (long)k);
    } else {
      ++k;
    }
  }
  if (in_flight) *in_flight = (int)s->active.size();
  if (queued) *queued = (int)s->queue.size();
  return NRSG_OK;
}

int nrsg_server_poll(nrsg_server *s, long long *request_id, nrsg_solve_info *info, int *got)
{
  if (!s || !request_id || !got) return NRSG_ERR_INVALID;
  std::lock_guard<std::mutex> lock(s->m);
  *got = 0;
  if (s->done.empty()) return NRSG_OK;
  *request_id = s->done.front().first;
  if (info) *info = s->done.front().second;
  const int code = s->doneCode.front();
  s->done.pop_front();
  s->doneCode.pop_front();
  *got = 1;
  return code == NRSG_ERR_MAXIT ? NRSG_OK : code;
}

} // extern "C"
