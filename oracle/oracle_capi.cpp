// ORACLE — test infrastructure only (see oracle_mesh.cpp header).
// Flat C entry points used by oracle/oracle.py (ctypes).
#include "oracle_internal.hpp"

#include <cmath>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>

using namespace orc;

namespace {
uint64_t splitmix64(uint64_t x)
{
  x += 0x9E3779B97F4A7C15ull;
  uint64_t z = x;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
} // namespace

extern "C" {

void orc_gll(int N, double *z, double *w) { gll(N, z, w); }
// weighted inner product sum_i w_i (a_i b_i) in the device's reduction order (w may be null: 1)
double orc_wdot(long long n, const double *w, const double *a, const double *b)
{
  if (!w)
    return wsum(n, [&](long long i, double &x, double &y) {
      x = a[i];
      y = b[i];
    });
  return wdot<double>(n, w, a, b);
}
// the fused PCG update: r = fma(-alpha, Ap, r), x = fma(alpha, p, x), returns (r, r)_w
double orc_update_pcg(long long n, const double *w, const double *p, const double *Ap, double alpha, double *x,
                      double *r)
{
  for (long long i = 0; i < n; ++i) {
    r[i] = std::fma(-alpha, Ap[i], r[i]);
    x[i] = std::fma(alpha, p[i], x[i]);
  }
  return wdot<double>(n, w, r, r);
}
void orc_dmatrix(int N, double *D)
{
  std::vector<double> z(N + 1), w(N + 1);
  gll(N, z.data(), w.data());
  dmatrix(N, z.data(), D);
}
void orc_interp(int Nin, int Nout, double *I)
{
  std::vector<double> zi(Nin + 1), wi(Nin + 1), zo(Nout + 1), wo(Nout + 1);
  gll(Nin, zi.data(), wi.data());
  gll(Nout, zo.data(), wo.data());
  interp_matrix(Nin + 1, zi.data(), Nout + 1, zo.data(), I);
}
void orc_box_mesh(int nx, int ny, int nz, double eps, double *VX, long long *EToV, int *EToB, int allDirichlet)
{
  box_mesh(nx, ny, nz, eps, VX, EToV, EToB, allDirichlet);
}
void orc_global_ids(int N, long long E, const long long *EToV, long long *ids) { global_ids(N, E, EToV, ids); }

// Seeded right-hand side for a box of nx*ny*nz elements: f is i.i.d.
// U[-1,1] per lattice node (splitmix64 of seed and the global lattice
// index), identical on every copy of a shared node; rhs = JW * f.
void orc_box_rhs(int N, int nx, int ny, int nz, unsigned long long seed, const double *ggeo, double *rhs)
{
  const int nq = N + 1, np = nq * nq * nq;
  const long long Lx = (long long)nx * N + 1, Ly = (long long)ny * N + 1;
  for (int ez = 0; ez < nz; ++ez)
    for (int ey = 0; ey < ny; ++ey)
      for (int ex = 0; ex < nx; ++ex) {
        const long long e = ex + (long long)nx * (ey + (long long)ny * ez);
        for (int k = 0; k < nq; ++k)
          for (int j = 0; j < nq; ++j)
            for (int i = 0; i < nq; ++i) {
              const long long g = (ex * N + i) + Lx * ((ey * N + j) + Ly * (long long)(ez * N + k));
              const uint64_t h = splitmix64(seed ^ splitmix64((uint64_t)g));
              const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);
              const int n = i + nq * (j + nq * k);
              rhs[e * np + n] = (2.0 * u - 1.0) * ggeo[e * 7 * np + 6 * np + n];
            }
      }
}

void *orc_create(int N, long long E, const double *VX, const long long *EToV, const int *EToB, const char *opts)
{
  try {
    auto *el = new Elliptic();
    el->setup(N, E, VX, EToV, EToB, opts ? opts : "");
    return el;
  } catch (const std::exception &ex) {
    fprintf(stderr, "oracle setup failed: %s\n", ex.what());
    return nullptr;
  }
}
void orc_destroy(void *h) { delete (Elliptic *)h; }

// named arrays of the fine level for parity tests
long long orc_size(void *h, const char *name)
{
  auto *el = (Elliptic *)h;
  const Level &L = el->fine;
  std::string s(name);
  if (s == "ids" || s == "maskedIds" || s == "x" || s == "y" || s == "z" || s == "invDegree") return L.Nlocal;
  if (s == "ggeo") return 7 * L.Nlocal;
  if (s == "gsOff") return (long long)L.gsOff.size();
  if (s == "gsIds") return (long long)L.gsIds.size();
  if (s == "maskIds") return (long long)L.maskIds.size();
  if (s == "invDiag") return (long long)el->invDiag.size();
  if (s == "D") return (long long)L.D.size();
  if (s == "history") return (long long)el->history.size();
  if (s == "allNeumann") return 1;
  return -1;
}
int orc_get(void *h, const char *name, void *out)
{
  auto *el = (Elliptic *)h;
  const Level &L = el->fine;
  std::string s(name);
  auto cp = [&](const auto &v) { std::memcpy(out, v.data(), v.size() * sizeof(v[0])); return 0; };
  if (s == "ids") return cp(L.ids);
  if (s == "maskedIds") return cp(L.maskedIds);
  if (s == "x") return cp(L.x);
  if (s == "y") return cp(L.y);
  if (s == "z") return cp(L.zc);
  if (s == "invDegree") return cp(L.invDegree);
  if (s == "ggeo") return cp(L.ggeo);
  if (s == "gsOff") return cp(L.gsOff);
  if (s == "gsIds") return cp(L.gsIds);
  if (s == "maskIds") return cp(L.maskIds);
  if (s == "invDiag") return cp(el->invDiag);
  if (s == "D") return cp(L.D);
  if (s == "history") return cp(el->history);
  if (s == "allNeumann") return cp(std::vector<double>{el->allNeumann ? 1.0 : 0.0});
  return -1;
}
double orc_volume(void *h) { return ((Elliptic *)h)->fine.volume; }

void orc_ax(void *h, const double *q, double *Aq) { ((Elliptic *)h)->ax(q, Aq); }
void orc_ax_ref(void *h, const double *q, double *Aq) { ((Elliptic *)h)->ax_ref(q, Aq); }
void orc_ax_fp32(void *h, const float *q, float *Aq)
{
  auto *el = (Elliptic *)h;
  const Level &L = el->fine;
  std::vector<float> g(L.ggeo.begin(), L.ggeo.end()), D(L.D.begin(), L.D.end());
  ax_stored<float>(L, g.data(), D.data(), (float)el->o.lambda0, (float)el->o.lambda1, el->o.poisson, q, Aq);
}
void orc_operator(void *h, const double *q, double *Aq) { ((Elliptic *)h)->op(q, Aq); }
void orc_gs(void *h, double *q) { gs_add(((Elliptic *)h)->fine, q); }
void orc_mask(void *h, double *q) { apply_mask(((Elliptic *)h)->fine, q); }
void orc_precond(void *h, const double *r, double *z) { ((Elliptic *)h)->precond(r, z); }

// rhs in (becomes the final residual), x in (x0) / out; info = {iters, res0, res, status}
int orc_solve(void *h, double *r, double *x, double *info)
{
  auto *el = (Elliptic *)h;
  double res0 = 0, res = 0;
  const int it = el->solve(r, x, res0, res);
  info[0] = it;
  info[1] = res0;
  info[2] = res;
  info[3] = el->status;
  return 0;
}

long long orc_mg_info(void *h, const char *what, double *out)
{
  auto v = mg_info(*(Elliptic *)h, what);
  if (out) std::memcpy(out, v.data(), v.size() * sizeof(double));
  return (long long)v.size();
}
long long orc_mg_level_size(void *h, int level) { return mg_level_size(*(Elliptic *)h, level); }
void orc_mg_schwarz(void *h, int level, const double *u, double *Su) { mg_level_smooth_schwarz(*(Elliptic *)h, level, u, Su); }

long long orc_mg_get(void *h, int level, const char *name, double *out)
{
  auto v = mg_level_array(*(Elliptic *)h, level, name);
  if (out) std::memcpy(out, v.data(), v.size() * sizeof(double));
  return (long long)v.size();
}
void orc_mg_transfer(void *h, int level, int restrict_, const double *in, double *out)
{
  mg_level_transfer(*(Elliptic *)h, level, restrict_ != 0, in, out);
}

double orc_hessenberg_rho(int n, const double *H) { return hessenberg_rho_public(n, H); }

// assembled fine-level operator (CSR); call with rowPtr == NULL for the sizes
void orc_assemble_fem(void *h, double lambda0, double lambda1, int poisson, long long *nrow, long long *nnz,
                      long long *rowPtr, long long *cols, double *vals)
{
  std::vector<long long> rp, c;
  std::vector<double> v;
  assemble_fem(((Elliptic *)h)->fine, lambda0, lambda1, poisson != 0, rp, c, v);
  *nrow = (long long)rp.size() - 1;
  *nnz = (long long)c.size();
  if (!rowPtr) return;
  std::memcpy(rowPtr, rp.data(), rp.size() * sizeof(long long));
  std::memcpy(cols, c.data(), c.size() * sizeof(long long));
  std::memcpy(vals, v.data(), v.size() * sizeof(double));
}

void orc_assemble_semfem(void *h, double lambda0, long long *nrow, long long *nnz, long long *rowPtr, long long *cols,
                         double *vals)
{
  std::vector<long long> rp, c;
  std::vector<double> v;
  assemble_semfem(((Elliptic *)h)->fine, lambda0, rp, c, v);
  *nrow = (long long)rp.size() - 1;
  *nnz = (long long)c.size();
  if (!rowPtr) return;
  std::memcpy(rowPtr, rp.data(), rp.size() * sizeof(long long));
  std::memcpy(cols, c.data(), c.size() * sizeof(long long));
  std::memcpy(vals, v.data(), v.size() * sizeof(double));
}

void orc_assemble_galerkin(void *hFine, void *hCoarse, double lambda0, double lambda1, int poisson, long long *nrow,
                           long long *nnz, long long *rowPtr, long long *cols, double *vals)
{
  std::vector<long long> rp, c;
  std::vector<double> v;
  assemble_galerkin(((Elliptic *)hFine)->fine, ((Elliptic *)hCoarse)->fine, lambda0, lambda1, poisson != 0, rp, c, v);
  *nrow = (long long)rp.size() - 1;
  *nnz = (long long)c.size();
  if (!rowPtr) return;
  std::memcpy(rowPtr, rp.data(), rp.size() * sizeof(long long));
  std::memcpy(cols, c.data(), c.size() * sizeof(long long));
  std::memcpy(vals, v.data(), v.size() * sizeof(double));
}

} // extern "C"
