#pragma once
#include <stddef.h>
int gsl_fit_linear(const double* x, size_t xs, const double* y, size_t ys, size_t n,
                   double* c0, double* c1, double* cov00, double* cov01, double* cov11, double* sumsq);
