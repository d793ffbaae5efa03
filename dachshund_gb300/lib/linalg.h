// Host BLAS-1 helpers with the reference's names (lib/linalg.h); c += a b
// and c -= a b elementwise.
#ifndef DS_GB300_CXX_LINALG_H
#define DS_GB300_CXX_LINALG_H

double ds_vector_dot(const int n, const double* const a, const double* const b);
double ds_vector_norm(const int n, const double* const x);
void ds_vector_add_cv(const int n, const double a, const double* const b, double* const c);
void ds_vector_sub_cv(const int n, const double a, const double* const b, double* const c);

#endif
