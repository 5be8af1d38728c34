// Exact weighted L1 regression on the host (shiftsSolver's objective,
// zorro_util.py:849-851: minimise sum_i w_i |(A x)_i - b_i|).
//
// The problem is solved through its dual linear programme
//     minimise  -b.y   subject to   A^T y = 0,   -w <= y <= w,
// which has only n equality rows (n = frames - 1) and m box-bounded
// variables (one per frame pair).  A bounded-variable revised simplex with an
// explicit n x n basis inverse does the work: phase 1 starts from every y at
// its lower bound with n artificial variables, phase 2 minimises -b.y.  At
// the optimum the simplex multipliers pi of the equality rows give the
// primal solution x = -pi, which fits the n basic pairs exactly.  Entering
// variables follow Dantzig's rule, switching to Bland's rule (smallest index)
// after a run of degenerate pivots so that the method cannot cycle.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "../../include/zorro_gb300.h"
#include "internal.h"

using namespace zr;

extern "C" int zr_l1_solve(const double* A, const double* b, const double* w, int m, int n, double lo, double hi,
                           double* x_out, int* status) {
  if (!A || !b || !w || !x_out || m <= 0 || n <= 0) return set_error(ZR_EINVAL, "zr_l1_solve: bad arguments");
  const int NV = m + n;
  const double tol = 1e-9, ptol = 1e-11;
  std::vector<double> lb(NV), ub(NV), val(NV), sgn(n), cost(NV);
  // Warm start: at the optimum every nonbasic y_j sits at -w_j sign(r_j),
  // r = A x - b.  Predict the signs from the weighted least-squares fit
  // (normal equations, Cholesky); the artificials of phase 1 absorb the rest.
  std::vector<double> x0(n, 0.0);
  {
    std::vector<double> N((size_t)n * n, 0.0), rhs(n, 0.0);
    for (int j = 0; j < m; j++) {
      const double wj = w[j] > 0.0 ? w[j] : 0.0;
      const double* aj = A + (size_t)j * n;
      for (int i = 0; i < n; i++) {
        if (aj[i] == 0.0) continue;
        rhs[i] += wj * aj[i] * b[j];
        for (int k = 0; k <= i; k++) N[(size_t)i * n + k] += wj * aj[i] * aj[k];
      }
    }
    bool ok = true;
    for (int i = 0; i < n && ok; i++) {
      for (int k = 0; k <= i; k++) {
        double s = N[(size_t)i * n + k];
        for (int q = 0; q < k; q++) s -= N[(size_t)i * n + q] * N[(size_t)k * n + q];
        if (i == k) {
          if (s <= 1e-12) { ok = false; break; }
          N[(size_t)i * n + i] = sqrt(s);
        } else {
          N[(size_t)i * n + k] = s / N[(size_t)k * n + k];
        }
      }
    }
    if (ok) {
      for (int i = 0; i < n; i++) {
        double s = rhs[i];
        for (int q = 0; q < i; q++) s -= N[(size_t)i * n + q] * x0[q];
        x0[i] = s / N[(size_t)i * n + i];
      }
      for (int i = n - 1; i >= 0; i--) {
        double s = x0[i];
        for (int q = i + 1; q < n; q++) s -= N[(size_t)q * n + i] * x0[q];
        x0[i] = s / N[(size_t)i * n + i];
      }
    } else {
      std::fill(x0.begin(), x0.end(), 0.0);
    }
  }
  for (int j = 0; j < m; j++) {
    const double wj = w[j] > 0.0 ? w[j] : 0.0;
    lb[j] = -wj;
    ub[j] = wj;
    double rj = -b[j];
    const double* aj = A + (size_t)j * n;
    for (int i = 0; i < n; i++) rj += aj[i] * x0[i];
    val[j] = rj > 0.0 ? -wj : wj;
  }
  // residual of A^T y = 0 at the starting point; artificials absorb it
  std::vector<double> r(n, 0.0);
  for (int j = 0; j < m; j++)
    for (int i = 0; i < n; i++) r[i] -= A[(size_t)j * n + i] * val[j];
  for (int i = 0; i < n; i++) {
    sgn[i] = r[i] >= 0.0 ? 1.0 : -1.0;
    lb[m + i] = 0.0;
    ub[m + i] = INFINITY;
    val[m + i] = fabs(r[i]);
  }
  std::vector<int> basis(n), where(NV, -1);
  std::vector<double> Binv((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) {
    basis[i] = m + i;
    where[m + i] = i;
    Binv[(size_t)i * n + i] = sgn[i];  // B = diag(sgn) is its own inverse
  }
  std::vector<double> a(n), alpha(n), pi(n), pre(n + 1, 0.0);
  // Rows that are one contiguous run of ones (pair (I, J) covers frames
  // I..J-1, the structure of zorro.py:1306-1311) price in O(1) from prefix
  // sums of pi.
  std::vector<int> r0(m, -1), r1(m, -1);
  bool runs = true;
  for (int j = 0; j < m && runs; j++) {
    const double* aj = A + (size_t)j * n;
    int first = -1, last = -1;
    for (int i = 0; i < n; i++) {
      if (aj[i] == 0.0) continue;
      if (aj[i] != 1.0 || (last >= 0 && i != last + 1)) { runs = false; break; }
      if (first < 0) first = i;
      last = i;
    }
    r0[j] = first;
    r1[j] = last + 1;
  }
  auto column = [&](int j, std::vector<double>& out) {
    if (j < m) {
      for (int i = 0; i < n; i++) out[i] = A[(size_t)j * n + i];
    } else {
      std::fill(out.begin(), out.end(), 0.0);
      out[j - m] = sgn[j - m];
    }
  };
  // Pricing state of every variable: act[j] = 1 for a nonbasic variable that
  // can move (0 for basic or fixed ones), up[j] = +1 at its upper bound, -1 at
  // its lower bound; the gain of moving it is up[j] * d_j (d_j its reduced
  // cost), so the pricing loop has no data-dependent branches.
  std::vector<double> act(NV), up(NV), rc(NV);
  auto set_state = [&](int j) {
    act[j] = (where[j] < 0 && ub[j] - lb[j] > 0.0) ? 1.0 : 0.0;
    up[j] = val[j] <= lb[j] ? -1.0 : 1.0;
  };
  auto compute_pi = [&]() {  // duals pi = c_B^T B^-1
    for (int k = 0; k < n; k++) {
      double s = 0.0;
      for (int i = 0; i < n; i++) s += cost[basis[i]] * Binv[(size_t)i * n + k];
      pi[k] = s;
    }
  };
  int iters = 0;
  const int max_iters = 50 * (m + n) + 1000;
  for (int phase = 1; phase <= 2; phase++) {
    for (int j = 0; j < NV; j++) cost[j] = (phase == 1) ? (j >= m ? 1.0 : 0.0) : (j < m ? -b[j] : 0.0);
    if (phase == 2) {
      // artificials are fixed at zero from here on
      for (int i = 0; i < n; i++) ub[m + i] = 0.0;
    }
    for (int j = 0; j < NV; j++) set_state(j);
    compute_pi();
    int degenerate_run = 0, since_refresh = 0;
    for (;;) {
      if (++iters > max_iters) {
        if (status) *status = 2;
        return set_error(ZR_EINVAL, "zr_l1_solve: iteration limit");
      }
      if (++since_refresh >= 32) {  // bound the drift of the updated duals
        compute_pi();
        since_refresh = 0;
      }
      // reduced costs
      if (runs) {
        pre[0] = 0.0;
        for (int k = 0; k < n; k++) pre[k + 1] = pre[k] + pi[k];
        for (int j = 0; j < m; j++) rc[j] = cost[j] - (r0[j] >= 0 ? pre[r1[j]] - pre[r0[j]] : 0.0);
      } else {
        for (int j = 0; j < m; j++) {
          double d = cost[j];
          const double* aj = A + (size_t)j * n;
          for (int i = 0; i < n; i++) d -= pi[i] * aj[i];
          rc[j] = d;
        }
      }
      for (int i = 0; i < n; i++) rc[m + i] = cost[m + i] - pi[i] * sgn[i];
      // entering variable: largest gain (Dantzig), or the first improving
      // variable (Bland) after a run of degenerate pivots
      const bool bland = degenerate_run > 50;
      int enter = -1;
      double best = tol;
      for (int j = 0; j < NV; j++) {
        const double gain = act[j] * up[j] * rc[j];
        if (gain > best) {
          enter = j;
          if (bland) break;
          best = gain;
        }
      }
      if (enter < 0) break;  // optimal for this phase
      const double dir = -up[enter];
      const double d_enter = rc[enter];
      if (runs && enter < m) {
        for (int i = 0; i < n; i++) {
          double s = 0.0;
          const double* bi = &Binv[(size_t)i * n];
          for (int k = r0[enter]; k < r1[enter]; k++) s += bi[k];
          alpha[i] = s;
        }
      } else {
        column(enter, a);
        for (int i = 0; i < n; i++) {
          double s = 0.0;
          for (int k = 0; k < n; k++) s += Binv[(size_t)i * n + k] * a[k];
          alpha[i] = s;
        }
      }
      // ratio test: x_B changes by -dir * alpha * t
      double tmax = ub[enter] - lb[enter];
      int leave = -1;
      double leave_to = 0.0;
      for (int i = 0; i < n; i++) {
        const double dlt = -dir * alpha[i];
        if (fabs(dlt) <= ptol) continue;
        const int bv = basis[i];
        double t;
        double bound;
        if (dlt < 0.0) { t = (val[bv] - lb[bv]) / -dlt; bound = lb[bv]; }
        else { if (isinf(ub[bv])) continue; t = (ub[bv] - val[bv]) / dlt; bound = ub[bv]; }
        if (t < 0.0) t = 0.0;
        if (t < tmax - 1e-15 || (leave >= 0 && fabs(t - tmax) <= 1e-15 && bv < basis[leave])) {
          tmax = t;
          leave = i;
          leave_to = bound;
        }
      }
      if (isinf(tmax)) {
        if (status) *status = 3;
        return set_error(ZR_EINVAL, "zr_l1_solve: unbounded (inconsistent weights)");
      }
      degenerate_run = (tmax <= 1e-12) ? degenerate_run + 1 : 0;
      for (int i = 0; i < n; i++) val[basis[i]] -= dir * alpha[i] * tmax;
      val[enter] += dir * tmax;
      if (leave < 0) {
        val[enter] = dir > 0 ? ub[enter] : lb[enter];  // bound flip
        set_state(enter);
        continue;
      }
      const int out = basis[leave];
      val[out] = leave_to;
      where[out] = -1;
      basis[leave] = enter;
      where[enter] = leave;
      set_state(out);
      set_state(enter);
      // B^-1 update with pivot alpha[leave]
      const double piv = alpha[leave];
      for (int k = 0; k < n; k++) Binv[(size_t)leave * n + k] /= piv;
      for (int i = 0; i < n; i++) {
        if (i == leave || alpha[i] == 0.0) continue;
        const double f = alpha[i];
        for (int k = 0; k < n; k++) Binv[(size_t)i * n + k] -= f * Binv[(size_t)leave * n + k];
      }
      // duals after the pivot: pi += d_enter * (new row `leave` of B^-1)
      for (int k = 0; k < n; k++) pi[k] += d_enter * Binv[(size_t)leave * n + k];
    }
    if (phase == 1) {
      double infeas = 0.0;
      for (int i = 0; i < n; i++) infeas += val[m + i];
      if (infeas > 1e-7) {
        if (status) *status = 1;
        return set_error(ZR_EINVAL, "zr_l1_solve: no feasible dual point");
      }
      // pivot remaining (zero-level) artificials out of the basis
      for (int i = 0; i < n; i++) {
        if (basis[i] < m) continue;
        int jbest = -1;
        double vbest = 1e-9;
        for (int j = 0; j < m; j++) {
          if (where[j] >= 0) continue;
          double s = 0.0;
          const double* aj = A + (size_t)j * n;
          for (int k = 0; k < n; k++) s += Binv[(size_t)i * n + k] * aj[k];
          if (fabs(s) > vbest) { vbest = fabs(s); jbest = j; }
        }
        if (jbest < 0) continue;  // redundant row
        column(jbest, a);
        for (int ii = 0; ii < n; ii++) {
          double s = 0.0;
          for (int k = 0; k < n; k++) s += Binv[(size_t)ii * n + k] * a[k];
          alpha[ii] = s;
        }
        const int out = basis[i];
        where[out] = -1;
        val[out] = 0.0;
        basis[i] = jbest;
        where[jbest] = i;
        const double piv = alpha[i];
        for (int k = 0; k < n; k++) Binv[(size_t)i * n + k] /= piv;
        for (int ii = 0; ii < n; ii++) {
          if (ii == i || alpha[ii] == 0.0) continue;
          const double f = alpha[ii];
          for (int k = 0; k < n; k++) Binv[(size_t)ii * n + k] -= f * Binv[(size_t)i * n + k];
        }
      }
    }
  }
  for (int k = 0; k < n; k++) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += cost[basis[i]] * Binv[(size_t)i * n + k];
    x_out[k] = -s;
  }
  int inside = 1;
  for (int k = 0; k < n; k++)
    if (x_out[k] < lo || x_out[k] > hi) inside = 0;
  if (status) *status = inside ? 0 : 4;
  return ZR_OK;
}
