/* TEST INFRASTRUCTURE (oracle build of the reference).  The reference links
 * -llapack -lblas (demonstrator/Makefile:36) for dgetrf_/dgetri_
 * (demonstrator/include/Helper.h:17,20).  No system LAPACK is installed here;
 * scipy's bundled OpenBLAS exports the same routines with a scipy_ prefix. */
void scipy_dgetrf_(int *M, int *N, double *A, int *lda, int *IPIV, int *INFO);
void scipy_dgetri_(int *N, double *A, int *lda, int *IPIV, double *WORK, int *lwork, int *INFO);
void dgetrf_(int *M, int *N, double *A, int *lda, int *IPIV, int *INFO) { scipy_dgetrf_(M, N, A, lda, IPIV, INFO); }
void dgetri_(int *N, double *A, int *lda, int *IPIV, double *WORK, int *lwork, int *INFO) { scipy_dgetri_(N, A, lda, IPIV, WORK, lwork, INFO); }
