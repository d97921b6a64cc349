/*
 * Host stand-in for the parts of SuiteSparse (CHOLMOD Core, SPQR) that the
 * reference's sparse_relax.cpp calls, used ONLY to compile that file for
 * pinning the oracle (see oracle/build_ref.sh).  SuiteSparse is not in this
 * image.  Matrices are stored dense (column-major) behind the CHOLMOD
 * types: the fixtures are a few hundred degrees of freedom.  The solve is
 * a dense least-squares solve standing in for SPQR's; for a full-rank
 * square system both give the unique solution.  The null-space helpers
 * (only reached with -n) abort.  Test infrastructure only.
 */
#ifndef NR_REFSHIM_SUITESPARSEQR_HPP
#define NR_REFSHIM_SUITESPARSEQR_HPP

#include <cstddef>
#include <cstring> /* the real headers bring <string.h> in; sparse_relax.cpp relies on it */

typedef long SuiteSparse_long;

enum { CHOLMOD_INT = 0, CHOLMOD_INTLONG = 1, CHOLMOD_LONG = 2 };
enum { CHOLMOD_PATTERN = 0, CHOLMOD_REAL = 1 };
#define SPQR_ORDERING_DEFAULT 7
#define SPQR_DEFAULT_TOL (-2)
#define SPQR_QX 0

struct cholmod_common {
    int useGPU;
    size_t gpuMemorySize;
};

struct cholmod_dense {
    size_t nrow, ncol, nzmax, d;
    void *x;
    int xtype;
};

struct cholmod_sparse {
    size_t nrow, ncol;
    int stype;
    double *a; /* nrow x ncol, column-major */
};

struct cholmod_triplet {
    size_t nrow, ncol, nzmax, nnz;
    void *i, *j, *x;
    int stype, itype, xtype;
};

int cholmod_l_start(cholmod_common *cc);
int cholmod_l_finish(cholmod_common *cc);
cholmod_triplet *cholmod_l_allocate_triplet(size_t nrow, size_t ncol, size_t nzmax, int stype, int xtype,
                                            cholmod_common *cc);
int cholmod_l_free_triplet(cholmod_triplet **T, cholmod_common *cc);
cholmod_sparse *cholmod_l_triplet_to_sparse(cholmod_triplet *T, size_t nzmax, cholmod_common *cc);
cholmod_sparse *cholmod_l_transpose(cholmod_sparse *A, int values, cholmod_common *cc);
cholmod_sparse *cholmod_l_ssmult(cholmod_sparse *A, cholmod_sparse *B, int stype, int values, int sorted,
                                 cholmod_common *cc);
int cholmod_l_free_sparse(cholmod_sparse **A, cholmod_common *cc);
cholmod_dense *cholmod_l_zeros(size_t nrow, size_t ncol, int xtype, cholmod_common *cc);
int cholmod_l_free_dense(cholmod_dense **X, cholmod_common *cc);
int cholmod_l_sdmult(cholmod_sparse *A, int transpose, double alpha[2], double beta[2], cholmod_dense *X,
                     cholmod_dense *Y, cholmod_common *cc);
int cholmod_l_copy_dense2(cholmod_dense *X, cholmod_dense *Y, cholmod_common *cc);
double cholmod_l_norm_dense(cholmod_dense *X, int norm, cholmod_common *cc);
int cholmod_l_print_sparse(cholmod_sparse *A, const char *name, cholmod_common *cc);
cholmod_sparse *cholmod_l_spzeros(size_t nrow, size_t ncol, size_t nzmax, int xtype, cholmod_common *cc);
cholmod_sparse *cholmod_l_speye(size_t nrow, size_t ncol, int xtype, cholmod_common *cc);
cholmod_sparse *cholmod_l_vertcat(cholmod_sparse *A, cholmod_sparse *B, int values, cholmod_common *cc);
cholmod_sparse *cholmod_l_horzcat(cholmod_sparse *A, cholmod_sparse *B, int values, cholmod_common *cc);
cholmod_sparse *cholmod_l_submatrix(cholmod_sparse *A, SuiteSparse_long *rset, SuiteSparse_long rsize,
                                    SuiteSparse_long *cset, SuiteSparse_long csize, int values, int sorted,
                                    cholmod_common *cc);

template <typename T>
struct SuiteSparseQR_factorization {
    SuiteSparse_long rank;
};
template <typename T>
cholmod_dense *SuiteSparseQR(cholmod_sparse *A, cholmod_dense *B, cholmod_common *cc);
template <typename T>
SuiteSparseQR_factorization<T> *SuiteSparseQR_factorize(int ordering, double tol, cholmod_sparse *A,
                                                        cholmod_common *cc);
template <typename T>
cholmod_sparse *SuiteSparseQR_qmult(int method, SuiteSparseQR_factorization<T> *QR, cholmod_sparse *X,
                                    cholmod_common *cc);
template <typename T>
void SuiteSparseQR_free(SuiteSparseQR_factorization<T> **QR, cholmod_common *cc);

template <>
cholmod_dense *SuiteSparseQR<double>(cholmod_sparse *A, cholmod_dense *B, cholmod_common *cc);
template <>
SuiteSparseQR_factorization<double> *SuiteSparseQR_factorize<double>(int ordering, double tol, cholmod_sparse *A,
                                                                     cholmod_common *cc);
template <>
cholmod_sparse *SuiteSparseQR_qmult<double>(int method, SuiteSparseQR_factorization<double> *QR, cholmod_sparse *X,
                                            cholmod_common *cc);
template <>
void SuiteSparseQR_free<double>(SuiteSparseQR_factorization<double> **QR, cholmod_common *cc);

#endif
