// Minimal stand-in for GSL's piecewise-linear spline (gsl_interp_linear).
// Index search: the largest i with x[i] <= x (bisection, clamped to n-2),
// then y = y[i] + (x - x[i]) / (x[i+1] - x[i]) * (y[i+1] - y[i]), the
// textbook linear interpolant GSL documents for gsl_interp_linear.
// Out-of-range x aborts, as GSL's default error handler does.
#pragma once
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <vector>

struct gsl_interp_type { int kind; };
static const gsl_interp_type gsl_interp_linear_value = {1};
static const gsl_interp_type* gsl_interp_linear = &gsl_interp_linear_value;

struct gsl_interp_accel { size_t cache; };
struct gsl_spline { std::vector<double> x, y; };

inline gsl_interp_accel* gsl_interp_accel_alloc() { return new gsl_interp_accel{0}; }
inline void gsl_interp_accel_free(gsl_interp_accel* a) { delete a; }
inline gsl_spline* gsl_spline_alloc(const gsl_interp_type*, size_t n) {
  gsl_spline* s = new gsl_spline;
  s->x.resize(n);
  s->y.resize(n);
  return s;
}
inline int gsl_spline_init(gsl_spline* s, const double* x, const double* y, size_t n) {
  s->x.assign(x, x + n);
  s->y.assign(y, y + n);
  return 0;
}
inline void gsl_spline_free(gsl_spline* s) { delete s; }
inline double gsl_spline_eval(const gsl_spline* s, double x, gsl_interp_accel*) {
  const size_t n = s->x.size();
  if (n < 2 || x < s->x[0] || x > s->x[n - 1]) {
    std::fprintf(stderr, "gsl shim: interpolation point %g out of range\n", x);
    std::abort();
  }
  size_t lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    size_t mid = (hi + lo) / 2;
    if (s->x[mid] > x) hi = mid; else lo = mid;
  }
  const double xl = s->x[lo], xh = s->x[lo + 1];
  const double yl = s->y[lo], yh = s->y[lo + 1];
  const double dx = xh - xl;
  return yl + (x - xl) / dx * (yh - yl);
}
