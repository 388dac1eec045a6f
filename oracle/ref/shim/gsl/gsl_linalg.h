/*
 * Declarations of the GSL symbols the reference names outside its hot path
 * (MLS, least squares and set-up RNG, sph.h:344-391, 994-1144, misc.cpp).
 * Test infrastructure for building the reference as a CPU checker: any call
 * aborts, so a run that strays off the hot path fails loudly.
 */
#ifndef ORACLE_SHIM_GSL_H
#define ORACLE_SHIM_GSL_H
#include <cstdlib>
struct gsl_matrix { int unused; };
struct gsl_vector { int unused; };
struct gsl_permutation { int unused; };
struct gsl_multifit_linear_workspace { int unused; };
struct gsl_rng { int unused; };
struct gsl_rng_type { int unused; };
struct gsl_eigen_symmv_workspace { int unused; };
struct gsl_matrix_view { gsl_matrix matrix; };
struct gsl_vector_view { gsl_vector vector; };
static const gsl_rng_type *gsl_rng_ranlxd1 = 0;
#define GSL_EIGEN_SORT_ABS_ASC 0
#define ORACLE_GSL_ABORT { std::abort(); }
inline gsl_matrix *gsl_matrix_alloc(int, int) ORACLE_GSL_ABORT
inline void gsl_matrix_free(gsl_matrix *) ORACLE_GSL_ABORT
inline void gsl_matrix_set_all(gsl_matrix *, double) ORACLE_GSL_ABORT
inline void gsl_matrix_set(gsl_matrix *, int, int, double) ORACLE_GSL_ABORT
inline double gsl_matrix_get(const gsl_matrix *, int, int) ORACLE_GSL_ABORT
inline gsl_vector *gsl_vector_alloc(int) ORACLE_GSL_ABORT
inline void gsl_vector_free(gsl_vector *) ORACLE_GSL_ABORT
inline void gsl_vector_set(gsl_vector *, int, double) ORACLE_GSL_ABORT
inline double gsl_vector_get(const gsl_vector *, int) ORACLE_GSL_ABORT
inline gsl_permutation *gsl_permutation_alloc(int) ORACLE_GSL_ABORT
inline void gsl_permutation_free(gsl_permutation *) ORACLE_GSL_ABORT
inline int gsl_linalg_LU_decomp(gsl_matrix *, gsl_permutation *, int *) ORACLE_GSL_ABORT
inline int gsl_linalg_LU_invert(const gsl_matrix *, const gsl_permutation *, gsl_matrix *) ORACLE_GSL_ABORT
inline gsl_multifit_linear_workspace *gsl_multifit_linear_alloc(int, int) ORACLE_GSL_ABORT
inline void gsl_multifit_linear_free(gsl_multifit_linear_workspace *) ORACLE_GSL_ABORT
inline int gsl_multifit_linear(const gsl_matrix *, const gsl_vector *, gsl_vector *, gsl_matrix *, double *, gsl_multifit_linear_workspace *) ORACLE_GSL_ABORT
inline gsl_rng *gsl_rng_alloc(const gsl_rng_type *) ORACLE_GSL_ABORT
inline void gsl_rng_set(gsl_rng *, unsigned long) ORACLE_GSL_ABORT
inline void gsl_rng_free(gsl_rng *) ORACLE_GSL_ABORT
inline double gsl_rng_uniform(gsl_rng *) ORACLE_GSL_ABORT
inline double gsl_ran_flat(gsl_rng *, double, double) ORACLE_GSL_ABORT
inline gsl_matrix_view gsl_matrix_view_array(double *, int, int) ORACLE_GSL_ABORT
inline gsl_vector_view gsl_matrix_column(gsl_matrix *, int) ORACLE_GSL_ABORT
inline gsl_eigen_symmv_workspace *gsl_eigen_symmv_alloc(int) ORACLE_GSL_ABORT
inline void gsl_eigen_symmv_free(gsl_eigen_symmv_workspace *) ORACLE_GSL_ABORT
inline int gsl_eigen_symmv(gsl_matrix *, gsl_vector *, gsl_matrix *, gsl_eigen_symmv_workspace *) ORACLE_GSL_ABORT
inline int gsl_eigen_symmv_sort(gsl_vector *, gsl_matrix *, int) ORACLE_GSL_ABORT
#endif
