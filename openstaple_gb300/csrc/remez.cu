// remez.cu -- the library's own generator of the rational approximations the
// RHMC reads from .REMEZ files (host code).  The reference produces them with
// an offline program over GMP multiprecision arithmetic
// (RationalApprox/rationalapprox_calc.cc, RationalApprox/Remez/alg_remez.cc);
// this is a new implementation of the same mathematical object, the best
// uniform approximation in relative error
//
//     r = P/Q of degree (n, n),   minimise max_{x in [lambda_min, 1]} |r(x)/x^b - 1|,
//
// of x^b with b = |num/den| in (0, 1), written as r(x) = a0 + sum_k a_k/(x + b_k)
// (positive exponent) or 1/r(x) = a0 + sum_k a_k/(x + b_k) (negative
// exponent, the reference's getIPFE convention), with the order loop of the
// reference's driver: a guessed order log(goal) log(lambda_min)/19 + 2, raised
// by one until the error is below the goal.
//
// Method (classical second Remez algorithm, in a parametrisation chosen for
// double-width arithmetic instead of multiprecision):
// * r(x) = c prod_k (x + z_k) / prod_k (x + p_k) with log c, log z_k, log p_k
//   as the unknowns: the zeros and poles of the best approximation of x^b
//   (0 < b < 1) are real, negative and interlaced, so positive z_k, p_k over
//   several decades are represented exactly and the relative error is a
//   product of well-conditioned factors (no monomial coefficients);
// * a start from the zeros and poles of Zolotarev's explicit best
//   approximation of x^(1/2) (Jacobi elliptic functions), each zero-pole pair
//   re-spaced for the exponent b, improved by Levenberg-Marquardt on the
//   least-squares misfit of log(r/x^b) at log-spaced samples;
// * then the exchange: the 2n+2 alternating extrema of e = r/x^b - 1 (one per
//   run of constant sign, located on a log grid and refined by golden-section
//   search), and Newton's method on e(x_i) = (-1)^i s E for the 2n+1
//   parameters and the level E, until the largest |e| on the interval equals
//   E to a relative 1e-9;
// * the partial fractions from the product form: a0 = c, b_k = p_k,
//   a_k = c prod_j (z_j - p_k) / prod_{j != k} (p_j - p_k) (and the same with
//   zeros and poles exchanged, 1/c, for the inverse).
// All of it in long double (64-bit significand on x86, 113-bit on AArch64).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>
#include "runtime.cuh"
#include "../../include/ostaple_gb300.h"

namespace {

typedef long double LD;

struct Rat {
  int n = 0;
  LD b = 0;                  // the exponent approximated, 0 < b < 1
  std::vector<LD> th;        // [log c, log z_1..z_n, log p_1..p_n]
  std::vector<LD> z, p;      // exp of the logs, refreshed by sync()
  LD c = 1;
  void sync() {
    c = expl(th[0]);
    z.resize(n);
    p.resize(n);
    for (int k = 0; k < n; ++k) {
      z[k] = expl(th[1 + k]);
      p[k] = expl(th[1 + n + k]);
    }
  }
  // r(x) / x^b
  LD ratio(LD x) const {
    LD v = c * powl(x, -b);
    for (int k = 0; k < n; ++k) v *= (x + z[k]) / (x + p[k]);
    return v;
  }
  LD err(LD x) const { return ratio(x) - 1; }
  // d log(r/x^b) / d th, written into g (2n+1)
  void dlog(LD x, LD* g) const {
    g[0] = 1;
    for (int k = 0; k < n; ++k) {
      g[1 + k] = z[k] / (x + z[k]);
      g[1 + n + k] = -p[k] / (x + p[k]);
    }
  }
};

// Solves A x = y (m x m, row-major, overwritten) by Gaussian elimination with
// partial pivoting; false when singular.
bool solve(std::vector<LD>& A, std::vector<LD>& y, int m) {
  for (int col = 0; col < m; ++col) {
    int piv = col;
    for (int r = col + 1; r < m; ++r)
      if (fabsl(A[r * m + col]) > fabsl(A[piv * m + col])) piv = r;
    if (!(fabsl(A[piv * m + col]) > 0)) return false;
    if (piv != col) {
      for (int k = 0; k < m; ++k) std::swap(A[col * m + k], A[piv * m + k]);
      std::swap(y[col], y[piv]);
    }
    for (int r = col + 1; r < m; ++r) {
      const LD f = A[r * m + col] / A[col * m + col];
      if (f == 0) continue;
      for (int k = col; k < m; ++k) A[r * m + k] -= f * A[col * m + k];
      y[r] -= f * y[col];
    }
  }
  for (int r = m - 1; r >= 0; --r) {
    LD s = y[r];
    for (int k = r + 1; k < m; ++k) s -= A[r * m + k] * y[k];
    y[r] = s / A[r * m + r];
  }
  return true;
}

std::vector<LD> log_grid(LD lo, LD hi, int count) {
  std::vector<LD> g(count);
  const LD l0 = logl(lo), l1 = logl(hi);
  for (int i = 0; i < count; ++i) g[i] = expl(l0 + (l1 - l0) * LD(i) / LD(count - 1));
  g[0] = lo;
  g[count - 1] = hi;
  return g;
}

void least_squares(Rat& r, LD lo, LD hi, const std::vector<LD>* weights = nullptr);

// Jacobi sn and cn of argument u and parameter m = k^2 by the descending
// Landen (arithmetic-geometric mean) transformation, Abramowitz and Stegun
// 16.4; returns K(m) too.
void jacobi_sn_cn(LD u, LD m, LD* sn, LD* cn, LD* K) {
  LD a[40], c[40];
  a[0] = 1;
  LD b = sqrtl(1 - m);
  c[0] = sqrtl(m);
  int N = 0;
  while (fabsl(c[N]) > LD(1e-30) && N < 38) {
    a[N + 1] = (a[N] + b) / 2;
    c[N + 1] = (a[N] - b) / 2;
    b = sqrtl(a[N] * b);
    ++N;
  }
  *K = acosl(LD(-1)) / (2 * a[N]);
  LD phi = ldexpl(a[N] * u, N);
  for (int i = N; i > 0; --i) phi = (phi + asinl(c[i] / a[i] * sinl(phi))) / 2;
  *sn = sinl(phi);
  *cn = cosl(phi);
}

// Start: the zeros and poles of Zolotarev's best relative approximation of
// x^(1/2) on [lo, 1] of the same order (breakpoints lo sn^2/cn^2 of
// l K'/(2n+1), l = 1..2n, modulus sqrt(1 - lo); zeros at odd l, poles at even
// l), each zero-pole pair moved apart or together about its geometric mean
// so that the pair's log gap is the fraction b of the local period; then
// least squares.
void initial_guess(Rat& r, LD lo, LD hi) {
  const int n = r.n;
  r.th.assign(2 * n + 1, 0);
  const LD m = 1 - lo / hi;
  LD sn, cn, K;
  jacobi_sn_cn(0, m, &sn, &cn, &K);
  std::vector<LD> q(2 * n + 1);
  for (int l = 1; l <= 2 * n; ++l) {
    jacobi_sn_cn(l * K / (2 * n + 1), m, &sn, &cn, &K);
    q[l] = lo * sn * sn / (cn * cn);
  }
  for (int k = 1; k <= n; ++k) {
    const LD lz = logl(q[2 * k - 1]), lp = logl(q[2 * k]), mid = (lz + lp) / 2, half = lp - lz;
    r.th[k] = mid - r.b * half;
    r.th[n + k] = mid + r.b * half;
  }
  least_squares(r, lo, hi);
}

// Alternating extrema of e: one per run of constant sign on a log grid,
// refined by golden-section search on |e| within the grid neighbours.
std::vector<LD> alternating_extrema(const Rat& r, LD lo, LD hi, int want) {
  const std::vector<LD> xs = log_grid(lo, hi, 600 * (r.n + 1));
  const int ns = int(xs.size());
  std::vector<LD> es(ns);
  for (int i = 0; i < ns; ++i) es[i] = r.err(xs[i]);
  struct Ext {
    LD x, e;
  };
  std::vector<Ext> ext;
  int i = 0;
  while (i < ns) {
    const bool pos = es[i] >= 0;
    int best = i, j = i;
    while (j < ns && ((es[j] >= 0) == pos)) {
      if (fabsl(es[j]) > fabsl(es[best])) best = j;
      ++j;
    }
    LD xb = xs[best], eb = es[best];
    if (best > 0 && best < ns - 1) {   // golden section on log x in (x_{best-1}, x_{best+1})
      LD a = logl(xs[best - 1]), b2 = logl(xs[best + 1]);
      const LD gr = (sqrtl(5.0L) - 1) / 2;
      LD c1 = b2 - gr * (b2 - a), c2 = a + gr * (b2 - a);
      LD f1 = fabsl(r.err(expl(c1))), f2 = fabsl(r.err(expl(c2)));
      for (int it = 0; it < 80; ++it) {
        if (f1 > f2) {
          b2 = c2; c2 = c1; f2 = f1;
          c1 = b2 - gr * (b2 - a);
          f1 = fabsl(r.err(expl(c1)));
        } else {
          a = c1; c1 = c2; f1 = f2;
          c2 = a + gr * (b2 - a);
          f2 = fabsl(r.err(expl(c2)));
        }
      }
      const LD xm = expl((a + b2) / 2), em = r.err(xm);
      if (fabsl(em) > fabsl(eb) && ((em >= 0) == pos)) {
        xb = xm;
        eb = em;
      }
    }
    ext.push_back({xb, eb});
    i = j;
  }
  // more runs than wanted: drop the smaller end until the count fits
  while (int(ext.size()) > want) {
    if (fabsl(ext.front().e) < fabsl(ext.back().e)) ext.erase(ext.begin());
    else ext.pop_back();
  }
  std::vector<LD> out;
  for (const Ext& e : ext) out.push_back(e.x);
  return out;
}

LD max_abs_err(const Rat& r, const std::vector<LD>& pts) {
  LD m = 0;
  for (LD x : pts) m = std::max(m, fabsl(r.err(x)));
  return m;
}

// The rounding error of one evaluation of e (4n + 8 roundings).
LD rounding_level(int n) { return LD(4 * n + 8) * std::numeric_limits<LD>::epsilon(); }

// Newton's method on e(x_i) - s_i E = 0 at the reference points.
bool levelled_solve(Rat& r, const std::vector<LD>& pts, LD* E) {
  const int n = r.n, m = 2 * n + 2;
  std::vector<LD> s(m);
  const LD s0 = r.err(pts[0]) >= 0 ? 1 : -1;
  for (int i = 0; i < m; ++i) s[i] = (i % 2 == 0) ? s0 : -s0;
  LD e = 0;
  for (int i = 0; i < m; ++i) e += fabsl(r.err(pts[i]));
  e /= m;
  auto resid = [&](const Rat& q, LD lev, std::vector<LD>& F) {
    LD nrm = 0;
    for (int i = 0; i < m; ++i) {
      F[i] = q.err(pts[i]) - s[i] * lev;
      nrm += F[i] * F[i];
    }
    return nrm;
  };
  std::vector<LD> F(m), g(m), A(m * m);
  LD nrm = resid(r, e, F);
  for (int it = 0; it < 60; ++it) {
    for (int i = 0; i < m; ++i) {
      const LD q = r.ratio(pts[i]);
      r.dlog(pts[i], g.data());
      for (int a = 0; a < m - 1; ++a) A[i * m + a] = q * g[a];
      A[i * m + m - 1] = -s[i];
    }
    std::vector<LD> y(m);
    for (int i = 0; i < m; ++i) y[i] = -F[i];
    std::vector<LD> M = A;
    if (!solve(M, y, m)) return false;
    LD step = 1;
    bool ok = false;
    for (int h = 0; h < 30; ++h, step /= 2) {
      Rat t = r;
      for (int a = 0; a < m - 1; ++a) t.th[a] += step * y[a];
      t.sync();
      const LD et = e + step * y[m - 1];
      std::vector<LD> Ft(m);
      const LD nt = resid(t, et, Ft);
      if (nt < nrm || nt == 0) {
        r = t;
        e = et;
        F = Ft;
        ok = nt < nrm * LD(0.999999) ;
        nrm = nt;
        break;
      }
    }
    if (!ok || nrm <= LD(1e-60) * (1 + e * e)) break;
  }
  *E = fabsl(e);
  return std::isfinite(double(*E));
}

// Least-squares fit of log(r / x^b) at log-spaced samples by
// Levenberg-Marquardt, from the parameters in r.
void least_squares(Rat& r, LD lo, LD hi, const std::vector<LD>* weights) {
  const int n = r.n, m = 2 * n + 1;
  const std::vector<LD> xs = log_grid(lo, hi, 40 * n + 40);
  const std::vector<LD> unit(xs.size(), LD(1));
  const std::vector<LD>& w = weights ? *weights : unit;
  auto cost = [&](const Rat& q) {
    LD s = 0;
    for (size_t j = 0; j < xs.size(); ++j) {
      const LD v = logl(q.ratio(xs[j]));
      s += w[j] * v * v;
    }
    return s;
  };
  r.sync();
  {   // c from the mean misfit
    LD s = 0;
    for (LD x : xs) s += logl(r.ratio(x));
    r.th[0] -= s / LD(xs.size());
    r.sync();
  }
  LD mu = 1e-3L, f0 = cost(r);
  std::vector<LD> g(m), JTJ(m * m), JTr(m);
  int quiet = 0;
  for (int it = 0; it < 200 && quiet < 3; ++it) {
    std::fill(JTJ.begin(), JTJ.end(), LD(0));
    std::fill(JTr.begin(), JTr.end(), LD(0));
    for (size_t j = 0; j < xs.size(); ++j) {
      const LD res = logl(r.ratio(xs[j]));
      r.dlog(xs[j], g.data());
      for (int a = 0; a < m; ++a) {
        JTr[a] += w[j] * g[a] * res;
        for (int b2 = 0; b2 < m; ++b2) JTJ[a * m + b2] += w[j] * g[a] * g[b2];
      }
    }
    bool improved = false;
    for (int tries = 0; tries < 20 && !improved; ++tries) {
      std::vector<LD> A = JTJ, y(m);
      for (int a = 0; a < m; ++a) {
        A[a * m + a] += mu * (JTJ[a * m + a] + LD(1e-30));
        y[a] = -JTr[a];
      }
      if (!solve(A, y, m)) {
        mu *= 4;
        continue;
      }
      Rat t = r;
      for (int a = 0; a < m; ++a) t.th[a] += y[a];
      t.sync();
      const LD f1 = cost(t);
      if (f1 < f0) {
        quiet = (f0 - f1) < LD(1e-10) * f0 ? quiet + 1 : 0;
        r = t;
        f0 = f1;
        mu = std::max(mu / 3, LD(1e-15));
        improved = true;
      } else {
        mu *= 4;
      }
    }
    if (!improved) return;
  }
}

// The exchange from the parameters in r; returns the error (negative when it
// fails).
double exchange(Rat& r, LD lo, LD hi) {
  const int want = 2 * r.n + 2;
  LD E = 0, best_err = 1e30L;
  Rat best = r;
  for (int it = 0; it < 80; ++it) {
    const std::vector<LD> pts = alternating_extrema(r, lo, hi, want);
    const LD mx = max_abs_err(r, pts);
    if (mx < best_err) {
      best_err = mx;
      best = r;
    }
    if (int(pts.size()) < want) return -1;   // not enough alternation from this start
    if (it > 0 && (mx - E) <= std::max(LD(1e-9) * E, LD(4) * rounding_level(r.n))) break;
    Rat t = r;
    if (!levelled_solve(t, pts, &E)) return -2;
    r = t;
  }
  const std::vector<LD> pts = alternating_extrema(r, lo, hi, want);
  const LD mx = max_abs_err(r, pts);
  if (mx > best_err) {
    r = best;
    return double(best_err);
  }
  return double(mx);
}

// Best approximation of x^b on [lo, hi] of order n; returns its error
// (negative when the exchange fails).
double remez(Rat& r, LD lo, LD hi) {
  initial_guess(r, lo, hi);
  // an order whose error lies near the rounding level of the arithmetic (far
  // below what double coefficients carry) cannot be levelled
  if (max_abs_err(r, alternating_extrema(r, lo, hi, 2 * r.n + 2)) < LD(1e4) * rounding_level(r.n)) return -3;
  Rat start = r;
  double e = exchange(r, lo, hi);
  // the least-squares start without the full alternation: Lawson's
  // reweighting (weights times |log(r/x^b)| at the samples) moves the fit
  // towards the minimax one, whose error alternates 2n+2 times
  const std::vector<LD> xs = log_grid(lo, hi, 40 * r.n + 40);
  std::vector<LD> w(xs.size(), LD(1) / LD(xs.size()));
  for (int round = 0; round < 12 && !(e > 0); ++round) {
    r = start;
    LD tot = 0;
    for (size_t j = 0; j < xs.size(); ++j) {
      w[j] *= fabsl(logl(r.ratio(xs[j])));
      tot += w[j];
    }
    if (!(tot > 0)) break;
    for (LD& v : w) v /= tot;
    least_squares(r, lo, hi, &w);
    start = r;
    if (int(alternating_extrema(r, lo, hi, 2 * r.n + 2).size()) >= 2 * r.n + 2) e = exchange(r, lo, hi);
  }
  return e;
}

// a0 + sum a_k / (x + b_k) of c prod (x + zz_k) / prod (x + pp_k), poles ascending
void partial_fractions(LD c, const std::vector<LD>& zz, const std::vector<LD>& pp, RationalApprox* out) {
  const int n = int(pp.size());
  std::vector<int> order(n);
  for (int k = 0; k < n; ++k) order[k] = k;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return pp[a] < pp[b]; });
  out->RA_a0 = double(c);
  for (int i = 0; i < n; ++i) {
    const int k = order[i];
    LD a = c;
    for (int j = 0; j < n; ++j) {
      a *= (zz[j] - pp[k]);
      if (j != k) a /= (pp[j] - pp[k]);
    }
    out->RA_a[i] = double(a);
    out->RA_b[i] = double(pp[k]);
  }
}

}  // namespace

extern "C" {

int ostaple_remez_approximation(RationalApprox* approx) {
  using ost::set_error;
  if (!approx) return -3;
  const int num = approx->exponent_num, den = approx->exponent_den, n = approx->approx_order;
  if (den == 0 || num == 0 || std::abs(num) >= std::abs(den)) {
    set_error(-3, "ostaple_remez_approximation: exponent %d/%d outside 0 < |num/den| < 1", num, den);
    return -3;
  }
  if (n < 1 || n > MAX_APPROX_ORDER) {
    set_error(-3, "ostaple_remez_approximation: order %d outside 1..%d", n, MAX_APPROX_ORDER);
    return -3;
  }
  if (!(approx->lambda_min > 0 && approx->lambda_min < 1)) {
    set_error(-3, "ostaple_remez_approximation: lambda_min %g outside (0, 1)", approx->lambda_min);
    return -3;
  }
  Rat r;
  r.n = n;
  r.b = LD(std::abs(num)) / LD(std::abs(den));
  const double e = remez(r, LD(approx->lambda_min), LD(1));
  if (e == -3) {
    set_error(-16, "ostaple_remez_approximation: the error of order %d for x^(%d/%d) on [%g, 1] is below the "
              "arithmetic's resolution; use a lower order", n, num, den, approx->lambda_min);
    return -16;
  }
  if (!(e > 0)) {
    set_error(-15, "ostaple_remez_approximation: the exchange did not converge (order %d, x^(%d/%d) on [%g, 1])", n,
              num, den, approx->lambda_min);
    return -15;
  }
  approx->lambda_max = 1.0;
  approx->gmp_remez_precision = 0;   // no multiprecision: long double arithmetic
  approx->error = e;
  for (int k = 0; k < MAX_APPROX_ORDER; ++k) approx->RA_a[k] = approx->RA_b[k] = 0.0;
  if (num * den > 0) partial_fractions(r.c, r.z, r.p, approx);
  else partial_fractions(1 / r.c, r.p, r.z, approx);
  return 0;
}

int ostaple_remez_generate(RationalApprox* approx, double goal_error, int fixed_order) {
  if (!approx || !(goal_error > 0)) return -3;
  // the reference driver's first guess of the order (rationalapprox_calc.cc)
  approx->approx_order = fixed_order > 0 ? fixed_order : int(log(goal_error) * log(approx->lambda_min) / 19 + 2);
  if (approx->approx_order < 1) approx->approx_order = 1;
  approx->error = 1;
  while (approx->error > goal_error) {
    const int rc = ostaple_remez_approximation(approx);
    if (rc != 0) return rc;
    if (approx->error > goal_error) {
      if (approx->approx_order >= MAX_APPROX_ORDER) {
        ost::set_error(-15, "ostaple_remez_generate: error %g above %g at the largest order %d", approx->error,
                       goal_error, MAX_APPROX_ORDER);
        return -15;
      }
      approx->approx_order++;
    }
  }
  return 0;
}

}  // extern "C"
