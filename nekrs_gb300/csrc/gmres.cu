// Restarted (flexible) GMRES on the device, restating PGMRES.cpp:111-340 and
// gmresUpdate (PGMRES.cpp:70-107): classical Gram-Schmidt through one fused
// weighted multi-dot and one fused orthogonalise+norm launch per step; the
// (nr+1)^2 Hessenberg and its Givens rotations stay on the host, which reads
// i+2 doubles per step.

#include "elliptic.hpp"

#include <cmath>

namespace nrsg {

void Elliptic::gmres_setup()
{
  const int nr = opt.nVector;
  if (nr < 1 || nr > 64) throw Error(NRSG_ERR_BAD_CONFIG, "nVector must be 1..64");
  const long long n = nT();
  const bool flexible = (opt.solver == "pfgmres");
  gV.alloc((size_t)nr * n);
  gZ.alloc((size_t)(flexible ? nr : 1) * n);
  gW.alloc(n);
  gB.alloc(n);
  gY.alloc(nr + 2);
  NRSG_CUDA(cudaMallocHost((void **)&h_y, sizeof(double) * (nr + 2)));
}

int Elliptic::pgmres(double *r, double *x, double tol, int maxit, double &rdotr)
{
  const long long n = nT();
  const double *wt = wT();
  const int nr = opt.nVector;
  const int ld = nr + 1;
  const bool flexible = (opt.solver == "pfgmres");
  std::vector<double> H((size_t)ld * ld, 0.0), sn(nr), cs(nr), s(nr + 1), y(nr);
  const double sqrtFac = std::sqrt(1.0 / fine.volume);
  NRSG_CUDA(cudaMemcpyAsync(gB.p, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
  double nrm = rdotr / sqrtFac;
  double error = rdotr;
  auto V = [&](int k) { return gV.p + (size_t)k * n; };
  auto Z = [&](int k) { return gZ.p + (size_t)(flexible ? k : 0) * n; };

  auto update = [&](int m) {
    for (int k = m - 1; k >= 0; --k) {
      y[k] = s[k];
      for (int j = k + 1; j < m; ++j) y[k] -= H[k + j * ld] * y[j];
      y[k] /= H[k + k * ld];
    }
    NRSG_CUDA(cudaMemcpyAsync(gY.p, y.data(), sizeof(double) * m, cudaMemcpyHostToDevice, stream));
    if (flexible) {
      launch_gmres_update(n, gZ.p, m, gY.p, x, stream);
    } else {
      launch_fill<double>(n, 0.0, z.p, stream);
      launch_gmres_update(n, gV.p, m, gY.p, z.p, stream);
      precondition(z.p, p.p);
      launch_axpby<double>(n, 1.0, p.p, 1.0, x, stream);
    }
    // y is consumed before the host buffer is reused
    NRSG_CUDA(cudaStreamSynchronize(stream));
  };

  int iter = 0;
  for (iter = 0; iter < maxit;) {
    s[0] = nrm;
    launch_scale_copy<double>(n, 1.0 / nrm, r, V(0), stream);
    for (int i = 0; i < nr; ++i) {
      double *Mv = Z(i);
      precondition(V(i), Mv);
      op(Mv, gW.p);
      launch_multi_wdot(n, wt, gV.p, i + 1, gW.p, gY.p, red, 0, stream);
      launch_gram_schmidt(n, wt, gV.p, i + 1, gY.p, gW.p, gY.p + nr + 1, red, 1, stream);
      NRSG_CUDA(cudaMemcpyAsync(h_y, gY.p, sizeof(double) * (nr + 2), cudaMemcpyDeviceToHost, stream));
      NRSG_CUDA(cudaStreamSynchronize(stream));
      const double nw = std::sqrt(h_y[nr + 1]);
      H[i + 1 + i * ld] = nw;
      if (i < nr - 1) launch_scale_copy<double>(n, 1.0 / nw, gW.p, V(i + 1), stream);
      for (int k = 0; k <= i; ++k) H[k + i * ld] = h_y[k];
      for (int k = 0; k < i; ++k) {
        const double h1 = H[k + i * ld], h2 = H[k + 1 + i * ld];
        H[k + i * ld] = cs[k] * h1 + sn[k] * h2;
        H[k + 1 + i * ld] = -sn[k] * h1 + cs[k] * h2;
      }
      const double h1 = H[i + i * ld], h2 = H[i + 1 + i * ld];
      const double hr = std::sqrt(h1 * h1 + h2 * h2);
      cs[i] = h1 / hr;
      sn[i] = h2 / hr;
      H[i + i * ld] = cs[i] * h1 + sn[i] * h2;
      H[i + 1 + i * ld] = 0;
      s[i + 1] = -sn[i] * s[i];
      s[i] = cs[i] * s[i];
      ++iter;
      error = std::fabs(s[i + 1]) * sqrtFac;
      rdotr = error;
      history.push_back(error);
      if (!std::isfinite(error)) {
        status = NRSG_ERR_NAN;
        return iter;
      }
      if (hr == 0.0) {
        status = NRSG_ERR_BREAKDOWN;
        return iter;
      }
      if (error < tol || iter == maxit) {
        update(i + 1);
        break;
      }
    }
    if (error < tol || iter == maxit) break;
    update(nr);
    op(x, Ap.p);
    launch_residual_norm(n, wt, gB.p, Ap.p, r, &d_scal.p->rdotr, red, 2, stream);
    nrm = std::sqrt(read_scalar(&d_scal.p->rdotr));
    error = nrm * sqrtFac;
    rdotr = error;
    if (error <= tol) return iter;
  }
  return iter;
}

} // namespace nrsg
