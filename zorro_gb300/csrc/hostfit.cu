// Host-side logistic fit of the peak-significance CDF (cdfLogisticCurve,
// zorro.py:1981-2022), in C++ so that it runs without the Python
// interpreter lock and without per-call NumPy overhead.
//
// Objective (zorro_util.py:862-863, in float64):
//   f(x) = sum_i | cdf_i - (1 - 1 / (1 + exp(-x1 (x0 - h_i)))^x2 |
// summed in NumPy's pairwise order, so that the value is the one
// np.sum(np.abs(...)) returns where NumPy's exp and pow are the C library's.
//
// Minimiser: bounded Nelder-Mead, the method of scipy.optimize.minimize(
// method='Nelder-Mead', bounds=...) with its default coefficients (reflection
// 1, expansion 2, contraction 0.5, shrink 0.5), 5 % start simplex reflected
// into the box, every trial point clipped to the box, the same stopping tests
// and the same function-evaluation limit; ties in the vertex order are kept
// in their previous order (a stable sort).
#include <math.h>
#include <string.h>

#include "internal.h"
#include "../../include/zorro_gb300.h"

namespace zr {

// np.add.reduce of a contiguous float64 vector: eight running sums over
// blocks of at most 128 values, combined pairwise; longer vectors split in
// two at a multiple of 8.
static double pairwise_sum(const double* a, long long n) {
  if (n < 8) {
    double r = 0.0;
    for (long long i = 0; i < n; i++) r += a[i];
    return r;
  }
  if (n <= 128) {
    double r[8];
    for (int j = 0; j < 8; j++) r[j] = a[j];
    long long i = 8;
    for (; i < n - (n % 8); i += 8)
      for (int j = 0; j < 8; j++) r[j] += a[i + j];
    double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
    for (; i < n; i++) res += a[i];
    return res;
  }
  long long n2 = n / 2;
  n2 -= n2 % 8;
  return pairwise_sum(a, n2) + pairwise_sum(a + n2, n - n2);
}

struct LogisticObjective {
  const double* nh;  // -h_i
  const float* cdf;
  int n;
  double* buf;
  double operator()(const double* x) const {
    const double a = -x[1];
    for (int i = 0; i < n; i++) {
      const double model = 1.0 - 1.0 / pow(1.0 + exp(a * (nh[i] + x[0])), x[2]);
      buf[i] = fabs((double)cdf[i] - model);
    }
    return pairwise_sum(buf, n);
  }
};

}  // namespace zr

using namespace zr;

extern "C" int zr_logistic_fit(const double* h_sigma, const float* cdf, int nbins, const double* x0,
                               const double* lo, const double* hi, double xatol, double fatol, int maxiter,
                               int maxfev, double* x_out, double* f_out, int* n_eval) {
  if (!h_sigma || !cdf || !x0 || !lo || !hi || !x_out || nbins <= 0)
    return set_error(ZR_EINVAL, "zr_logistic_fit: null argument or no bins");
  constexpr int n = 3;
  for (int k = 0; k < n; k++)
    if (lo[k] > hi[k]) return set_error(ZR_EINVAL, "zr_logistic_fit: lower bound above upper bound");
  double* nh = new double[2 * (size_t)nbins];
  for (int i = 0; i < nbins; i++) nh[i] = -h_sigma[i];
  LogisticObjective f{nh, cdf, nbins, nh + nbins};

  auto clip = [&](double* p) {
    for (int k = 0; k < n; k++) p[k] = fmin(fmax(p[k], lo[k]), hi[k]);
  };
  double sim[n + 1][n], fs[n + 1];
  double start[n];
  for (int k = 0; k < n; k++) start[k] = x0[k];
  clip(start);
  for (int j = 0; j <= n; j++) memcpy(sim[j], start, sizeof(start));
  for (int k = 0; k < n; k++) sim[k + 1][k] = sim[k + 1][k] != 0.0 ? (1.0 + 0.05) * sim[k + 1][k] : 0.00025;
  for (int j = 0; j <= n; j++)
    for (int k = 0; k < n; k++) {
      double v = sim[j][k];
      if (v > hi[k]) v = 2.0 * hi[k] - v;
      sim[j][k] = fmin(fmax(v, lo[k]), hi[k]);
    }
  int calls = 0;
  bool out_of_calls = false;
  auto eval = [&](const double* p, double& fv) -> bool {
    if (calls >= maxfev) {
      out_of_calls = true;
      return false;
    }
    calls++;
    fv = f(p);
    return true;
  };
  auto order = [&]() {  // stable insertion sort of the vertices by value
    for (int i = 1; i <= n; i++) {
      double fv = fs[i], pv[n];
      memcpy(pv, sim[i], sizeof(pv));
      int j = i - 1;
      while (j >= 0 && fs[j] > fv) {
        fs[j + 1] = fs[j];
        memcpy(sim[j + 1], sim[j], sizeof(pv));
        j--;
      }
      fs[j + 1] = fv;
      memcpy(sim[j + 1], pv, sizeof(pv));
    }
  };
  for (int j = 0; j <= n; j++) fs[j] = INFINITY;
  for (int j = 0; j <= n; j++)
    if (!eval(sim[j], fs[j])) break;
  order();
  int it = 1;
  while (calls < maxfev && it < maxiter) {
    double dx = 0.0, df = 0.0;
    for (int i = 1; i <= n; i++) {
      for (int k = 0; k < n; k++) dx = fmax(dx, fabs(sim[i][k] - sim[0][k]));
      df = fmax(df, fabs(fs[0] - fs[i]));
    }
    if (dx <= xatol && df <= fatol) break;
    do {  // one iteration; a break leaves it when the evaluation limit is hit
      double xbar[n], xr[n], fxr;
      for (int k = 0; k < n; k++) {
        double acc = sim[0][k];
        for (int i = 1; i < n; i++) acc = acc + sim[i][k];
        xbar[k] = acc / n;
      }
      const double* last = sim[n];
      for (int k = 0; k < n; k++) xr[k] = 2.0 * xbar[k] - last[k];
      clip(xr);
      if (!eval(xr, fxr)) break;
      if (fxr < fs[0]) {
        double xe[n], fxe;
        for (int k = 0; k < n; k++) xe[k] = 3.0 * xbar[k] - 2.0 * last[k];
        clip(xe);
        if (!eval(xe, fxe)) break;
        if (fxe < fxr) {
          memcpy(sim[n], xe, sizeof(xe));
          fs[n] = fxe;
        } else {
          memcpy(sim[n], xr, sizeof(xr));
          fs[n] = fxr;
        }
      } else if (fxr < fs[n - 1]) {
        memcpy(sim[n], xr, sizeof(xr));
        fs[n] = fxr;
      } else {
        bool shrink = false;
        if (fxr < fs[n]) {
          double xc[n], fxc;
          for (int k = 0; k < n; k++) xc[k] = 1.5 * xbar[k] - 0.5 * last[k];
          clip(xc);
          if (!eval(xc, fxc)) break;
          if (fxc <= fxr) {
            memcpy(sim[n], xc, sizeof(xc));
            fs[n] = fxc;
          } else {
            shrink = true;
          }
        } else {
          double xcc[n], fxcc;
          for (int k = 0; k < n; k++) xcc[k] = 0.5 * xbar[k] + 0.5 * last[k];
          clip(xcc);
          if (!eval(xcc, fxcc)) break;
          if (fxcc < fs[n]) {
            memcpy(sim[n], xcc, sizeof(xcc));
            fs[n] = fxcc;
          } else {
            shrink = true;
          }
        }
        if (shrink) {
          bool stop = false;
          for (int j = 1; j <= n && !stop; j++) {
            for (int k = 0; k < n; k++) sim[j][k] = sim[0][k] + 0.5 * (sim[j][k] - sim[0][k]);
            clip(sim[j]);
            if (!eval(sim[j], fs[j])) stop = true;
          }
          if (stop) break;
        }
      }
      it++;
    } while (false);
    order();
    if (out_of_calls) break;
  }
  memcpy(x_out, sim[0], sizeof(double) * n);
  if (f_out) {
    double m = fs[0];
    for (int j = 1; j <= n; j++) m = fmin(m, fs[j]);
    *f_out = m;
  }
  if (n_eval) *n_eval = calls;
  delete[] nh;
  return ZR_OK;
}
