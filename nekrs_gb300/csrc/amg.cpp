// Classical algebraic multigrid for the coarsest p-multigrid level
// (coarseSolver = amg): the configuration the reference hands to BoomerAMG
// (hypre 2.28.0, a third-party library the reference vendors; its call site
// coarseLevel.cpp:77-133 sets coarsening 10 (HMIS), interpolation 6
// (extended+i), strength 0.25, one V-cycle, Chebyshev smoothing of order 1),
// restated from the published algorithms:
//   strength       j strongly influences i if -a_ij >= theta max_{k != i}(-a_ik)
//   coarsening     Ruge-Stueben first pass (HMIS on one process is its first
//                  pass): repeatedly the unassigned point influencing the most
//                  unassigned points (lowest index on ties) becomes C, the points
//                  it strongly influences F, and the points influencing those F
//                  points gain weight
//   interpolation  extended+i (De Sterck, Falgout, Nolting, Yang, Numer. Linear
//                  Algebra Appl. 15 (2008) 115-139): the interpolatory set of an
//                  F point is its strong C neighbours and the strong C neighbours
//                  of its strong F neighbours; each strong F neighbour k is
//                  distributed over that set and i itself through the entries of
//                  row k whose sign differs from a_kk; weak couplings outside the
//                  set are added to the diagonal; rows truncated to the 4 largest
//                  weights with the row sum kept (hypre's default P_max_elmts)
//   coarse ops     Galerkin R A P, R = P^T
//   smoothing      Chebyshev of degree 1 on D^-1 A over [0.3 lmax, lmax]:
//                  x += 2 / (1.3 lmax) D^-1 r, one sweep down and one up; lmax by
//                  Rayleigh quotients of the power iteration on D^-1/2 A D^-1/2
//   coarsest       dense inverse (Gaussian elimination, BoomerAMG's relaxation 9
//                  on its coarsest level)
#include "amg.hpp"

#include <algorithm>
#include <cmath>
#include <queue>

namespace nrsg {

namespace {

void strength(const AmgCsr &A, double theta, AmgCsr &S)
{
  S = AmgCsr();
  S.n = S.m = A.n;
  S.rp.assign((size_t)A.n + 1, 0);
  for (int i = 0; i < A.n; ++i) {
    double mx = 0;
    bool any = false;
    for (int q = A.rp[i]; q < A.rp[i + 1]; ++q)
      if (A.ci[q] != i) {
        if (!any || -A.v[q] > mx) mx = -A.v[q];
        any = true;
      }
    if (any && mx > 0)
      for (int q = A.rp[i]; q < A.rp[i + 1]; ++q)
        if (A.ci[q] != i && -A.v[q] >= theta * mx) S.ci.push_back(A.ci[q]);
    S.rp[i + 1] = (int)S.ci.size();
  }
  S.v.assign(S.ci.size(), 1.0);
}

void transpose_pattern(const AmgCsr &S, AmgCsr &T)
{
  T = AmgCsr();
  T.n = S.m;
  T.m = S.n;
  T.rp.assign((size_t)T.n + 1, 0);
  for (int c : S.ci) ++T.rp[c + 1];
  for (int i = 0; i < T.n; ++i) T.rp[i + 1] += T.rp[i];
  T.ci.resize(S.ci.size());
  std::vector<int> pos(T.rp.begin(), T.rp.end() - 1);
  for (int i = 0; i < S.n; ++i)
    for (int q = S.rp[i]; q < S.rp[i + 1]; ++q) T.ci[pos[S.ci[q]]++] = i;
}

// state: 1 C, -1 F
void rs_first_pass(const AmgCsr &S, std::vector<signed char> &state)
{
  const int n = S.n;
  AmgCsr ST;
  transpose_pattern(S, ST);
  std::vector<long long> lam(n);
  for (int i = 0; i < n; ++i) lam[i] = ST.rp[i + 1] - ST.rp[i];
  state.assign(n, 0);
  using Item = std::pair<long long, int>; // (-lambda, index): smallest first = largest lambda, lowest index
  std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
  for (int i = 0; i < n; ++i) heap.push({-lam[i], i});
  while (!heap.empty()) {
    const Item it = heap.top();
    heap.pop();
    const int i = it.second;
    if (state[i] != 0 || -it.first != lam[i]) continue;
    if (lam[i] == 0 && S.rp[i + 1] == S.rp[i]) {
      state[i] = -1;
      continue;
    }
    state[i] = 1;
    for (int q = ST.rp[i]; q < ST.rp[i + 1]; ++q) {
      const int j = ST.ci[q];
      if (state[j] != 0) continue;
      state[j] = -1;
      for (int r = S.rp[j]; r < S.rp[j + 1]; ++r) {
        const int k = S.ci[r];
        if (state[k] == 0) heap.push({-(++lam[k]), k});
      }
    }
    for (int q = S.rp[i]; q < S.rp[i + 1]; ++q) {
      const int k = S.ci[q];
      if (state[k] == 0) heap.push({-(--lam[k]), k});
    }
  }
  for (auto &s : state)
    if (s == 0) s = -1;
}

double row_entry(const AmgCsr &A, int i, int j)
{
  const int *b = A.ci.data() + A.rp[i], *e = A.ci.data() + A.rp[i + 1];
  const int *p = std::lower_bound(b, e, j);
  return (p != e && *p == j) ? A.v[(size_t)(p - A.ci.data())] : 0.0;
}

void ext_i_interp(const AmgCsr &A, const AmgCsr &S, const std::vector<signed char> &state, int pmax, AmgCsr &P)
{
  const int n = A.n;
  std::vector<int> cidx(n, -1);
  int nc = 0;
  for (int i = 0; i < n; ++i)
    if (state[i] == 1) cidx[i] = nc++;
  P = AmgCsr();
  P.n = n;
  P.m = nc;
  P.rp.assign((size_t)n + 1, 0);
  std::vector<char> inCt(n, 0), inFs(n, 0);
  std::vector<double> w(n, 0.0);
  std::vector<int> Ct, Fs;
  for (int i = 0; i < n; ++i) {
    if (state[i] == 1) {
      P.ci.push_back(cidx[i]);
      P.v.push_back(1.0);
      P.rp[i + 1] = (int)P.ci.size();
      continue;
    }
    Ct.clear();
    Fs.clear();
    for (int q = S.rp[i]; q < S.rp[i + 1]; ++q) {
      const int j = S.ci[q];
      if (state[j] == 1) {
        if (!inCt[j]) inCt[j] = 1, Ct.push_back(j);
      } else {
        Fs.push_back(j);
        inFs[j] = 1;
      }
    }
    for (int k : Fs)
      for (int q = S.rp[k]; q < S.rp[k + 1]; ++q) {
        const int j = S.ci[q];
        if (state[j] == 1 && !inCt[j]) inCt[j] = 1, Ct.push_back(j);
      }
    std::sort(Ct.begin(), Ct.end());
    if (!Ct.empty()) {
      double at = row_entry(A, i, i);
      for (int j : Ct) w[j] = row_entry(A, i, j);
      for (int q = A.rp[i]; q < A.rp[i + 1]; ++q) {
        const int j = A.ci[q];
        if (j == i || inCt[j] || inFs[j]) continue;
        at += A.v[q]; // weak couplings outside the interpolatory set
      }
      for (int k : Fs) {
        const double akk = row_entry(A, k, k);
        auto bar = [akk](double v) { return ((v < 0) != (akk < 0) && v != 0) ? v : 0.0; };
        double den = 0;
        for (int l : Ct) den += bar(row_entry(A, k, l));
        den += bar(row_entry(A, k, i));
        const double aik = row_entry(A, i, k);
        if (den == 0) {
          at += aik;
          continue;
        }
        for (int j : Ct) w[j] += aik * bar(row_entry(A, k, j)) / den;
        at += aik * bar(row_entry(A, k, i)) / den;
      }
      // weights, then truncation to the pmax largest |w| (stable on ties) with the row sum kept
      std::vector<std::pair<int, double>> row;
      row.reserve(Ct.size());
      for (int j : Ct) row.push_back({j, -w[j] / at});
      if (pmax > 0 && (int)row.size() > pmax) {
        double tot = 0;
        for (auto &p : row) tot += p.second;
        std::vector<int> ord(row.size());
        for (size_t q = 0; q < ord.size(); ++q) ord[q] = (int)q;
        std::stable_sort(ord.begin(), ord.end(),
                         [&](int a, int b) { return std::fabs(row[a].second) > std::fabs(row[b].second); });
        std::vector<std::pair<int, double>> kept;
        double ks = 0;
        for (int q = 0; q < pmax; ++q) kept.push_back(row[ord[q]]), ks += row[ord[q]].second;
        const double sc = ks != 0 ? tot / ks : 1.0;
        for (auto &p : kept) p.second *= sc;
        std::sort(kept.begin(), kept.end());
        row.swap(kept);
      }
      for (auto &p : row) {
        P.ci.push_back(cidx[p.first]);
        P.v.push_back(p.second);
      }
      for (int j : Ct) w[j] = 0.0;
    }
    for (int j : Ct) inCt[j] = 0;
    for (int k : Fs) inFs[k] = 0;
    P.rp[i + 1] = (int)P.ci.size();
  }
}

void transpose(const AmgCsr &P, AmgCsr &R)
{
  R = AmgCsr();
  R.n = P.m;
  R.m = P.n;
  R.rp.assign((size_t)R.n + 1, 0);
  for (int c : P.ci) ++R.rp[c + 1];
  for (int i = 0; i < R.n; ++i) R.rp[i + 1] += R.rp[i];
  R.ci.resize(P.ci.size());
  R.v.resize(P.ci.size());
  std::vector<int> pos(R.rp.begin(), R.rp.end() - 1);
  for (int i = 0; i < P.n; ++i)
    for (int q = P.rp[i]; q < P.rp[i + 1]; ++q) {
      const int d = pos[P.ci[q]]++;
      R.ci[d] = i;
      R.v[d] = P.v[q];
    }
}

// C = A B (Gustavson, columns of each row sorted, exact zeros dropped)
void spgemm(const AmgCsr &A, const AmgCsr &B, AmgCsr &C)
{
  C = AmgCsr();
  C.n = A.n;
  C.m = B.m;
  C.rp.assign((size_t)A.n + 1, 0);
  std::vector<int> mark(B.m, -1);
  std::vector<double> acc(B.m, 0.0);
  std::vector<int> cols;
  for (int i = 0; i < A.n; ++i) {
    cols.clear();
    for (int q = A.rp[i]; q < A.rp[i + 1]; ++q) {
      const int k = A.ci[q];
      const double a = A.v[q];
      for (int r = B.rp[k]; r < B.rp[k + 1]; ++r) {
        const int j = B.ci[r];
        if (mark[j] != i) mark[j] = i, acc[j] = 0.0, cols.push_back(j);
        acc[j] += a * B.v[r];
      }
    }
    std::sort(cols.begin(), cols.end());
    for (int j : cols)
      if (acc[j] != 0.0) C.ci.push_back(j), C.v.push_back(acc[j]);
    C.rp[i + 1] = (int)C.ci.size();
  }
}

// largest eigenvalue of D^-1 A (= that of D^-1/2 A D^-1/2): Rayleigh quotients of the power iteration
double lambda_max(const AmgCsr &A, const std::vector<double> &dinv)
{
  const int n = A.n;
  std::vector<double> x(n), y(n), s(n);
  for (int i = 0; i < n; ++i) s[i] = std::sqrt(dinv[i]);
  for (int i = 0; i < n; ++i) x[i] = 1.0 + 0.5 * std::sin(1.0 + 0.7 * i);
  double lam = 0;
  for (int it = 0; it < 60; ++it) {
    double nx = 0;
    for (int i = 0; i < n; ++i) nx += x[i] * x[i];
    nx = std::sqrt(nx);
    for (int i = 0; i < n; ++i) x[i] /= nx;
    double xy = 0;
    for (int i = 0; i < n; ++i) {
      double t = 0;
      for (int q = A.rp[i]; q < A.rp[i + 1]; ++q) t += A.v[q] * s[A.ci[q]] * x[A.ci[q]];
      y[i] = s[i] * t;
      xy += x[i] * y[i];
    }
    lam = xy;
    x.swap(y);
  }
  return lam;
}

// inverse of the dense n x n matrix of A (Gauss-Jordan, partial pivoting)
bool dense_inverse(const AmgCsr &A, std::vector<double> &inv)
{
  const int n = A.n;
  std::vector<double> M((size_t)n * n, 0.0);
  inv.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) {
    for (int q = A.rp[i]; q < A.rp[i + 1]; ++q) M[(size_t)i * n + A.ci[q]] = A.v[q];
    inv[(size_t)i * n + i] = 1.0;
  }
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(M[(size_t)r * n + c]) > std::fabs(M[(size_t)p * n + c])) p = r;
    if (M[(size_t)p * n + c] == 0.0) return false;
    if (p != c)
      for (int k = 0; k < n; ++k) {
        std::swap(M[(size_t)p * n + k], M[(size_t)c * n + k]);
        std::swap(inv[(size_t)p * n + k], inv[(size_t)c * n + k]);
      }
    const double d = 1.0 / M[(size_t)c * n + c];
    for (int k = 0; k < n; ++k) {
      M[(size_t)c * n + k] *= d;
      inv[(size_t)c * n + k] *= d;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = M[(size_t)r * n + c];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) {
        M[(size_t)r * n + k] -= f * M[(size_t)c * n + k];
        inv[(size_t)r * n + k] -= f * inv[(size_t)c * n + k];
      }
    }
  }
  return true;
}

} // namespace

void amg_build(long long n, const long long *rowPtr, const long long *col, const double *val, AmgHierarchy &H,
               const AmgParams &prm)
{
  H = AmgHierarchy();
  AmgCsr A;
  A.n = A.m = (int)n;
  A.rp.resize((size_t)n + 1);
  for (long long i = 0; i <= n; ++i) A.rp[i] = (int)rowPtr[i];
  A.ci.resize((size_t)A.rp[n]);
  A.v.resize((size_t)A.rp[n]);
  for (long long i = 0; i < n; ++i) {
    // rows sorted by column
    std::vector<std::pair<int, double>> row;
    for (long long q = rowPtr[i]; q < rowPtr[i + 1]; ++q) row.push_back({(int)col[q], val[q]});
    std::sort(row.begin(), row.end());
    for (size_t q = 0; q < row.size(); ++q) {
      A.ci[(size_t)rowPtr[i] + q] = row[q].first;
      A.v[(size_t)rowPtr[i] + q] = row[q].second;
    }
  }
  while (A.n > prm.maxCoarse && (int)H.levels.size() < prm.maxLevels) {
    AmgCsr S;
    strength(A, prm.theta, S);
    std::vector<signed char> state;
    rs_first_pass(S, state);
    int nc = 0;
    for (auto s : state) nc += s == 1;
    if (nc == 0 || nc == A.n) break;
    AmgLevelHost L;
    ext_i_interp(A, S, state, prm.pmax, L.P);
    transpose(L.P, L.R);
    L.dinv.resize(A.n);
    for (int i = 0; i < A.n; ++i) L.dinv[i] = 1.0 / row_entry(A, i, i);
    L.lmax = lambda_max(A, L.dinv);
    AmgCsr AP, Ac;
    spgemm(A, L.P, AP);
    spgemm(L.R, AP, Ac);
    L.A = std::move(A);
    H.levels.push_back(std::move(L));
    A = std::move(Ac);
  }
  H.coarse = std::move(A);
  H.invertible = dense_inverse(H.coarse, H.coarseInv);
}

} // namespace nrsg
