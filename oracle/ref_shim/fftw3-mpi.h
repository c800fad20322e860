/*
 * fftw3-mpi.h — ORACLE test infrastructure: a single-rank stand-in for the
 * subset of FFTW 3.3's MPI interface (fftw3-mpi.h with the fftw3.h types it
 * pulls in) that the reference's Solver/src/solver.c uses:
 *   fftw_mpi_local_size_3d / _many      (solver.c:1844-1845)
 *   fftw_mpi_plan_dft_{r2c,c2r}_3d      (solver.c:2045-2046)
 *   fftw_mpi_plan_many_dft_{r2c,c2r}    (solver.c:2056-2068)
 *   fftw_mpi_execute_dft_{r2c,c2r}      (solver.c:656, 658, 683, 1573, 1599)
 *   fftw_malloc / fftw_free / fftw_destroy_plan.
 * The transforms follow FFTW's documented conventions: unnormalised, the
 * advanced ("many") layout with howmany components interleaved, the real
 * array padded to 2 (n2/2 + 1) in the last dimension, and
 * FFTW_MPI_TRANSPOSED_IN / _OUT exchanging the first two dimensions of the
 * complex array. The 1D transforms are the oracle's own (orc_fft_plan_*).
 * FFTW itself is not vendored in the reference and not installed here.
 */
#ifndef NS3D_REF_SHIM_FFTW3_MPI_H
#define NS3D_REF_SHIM_FFTW3_MPI_H
#include <complex.h>
#include <stddef.h>

#include "mpi.h"

/* fftw3.h makes fftw_complex the C99 complex type when <complex.h> comes
   first, as it does in solver.c:14 and utils.c:15. */
typedef double _Complex fftw_complex;
typedef struct ns3d_ref_plan* fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_MPI_DEFAULT_BLOCK ((ptrdiff_t)0)
#define FFTW_MPI_TRANSPOSED_IN (1U << 29)
#define FFTW_MPI_TRANSPOSED_OUT (1U << 30)

void* fftw_malloc(size_t n);
void fftw_free(void* p);
void fftw_destroy_plan(fftw_plan p);
void fftw_mpi_init(void);
void fftw_mpi_cleanup(void);

ptrdiff_t fftw_mpi_local_size_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, MPI_Comm comm, ptrdiff_t* local_n0,
                                 ptrdiff_t* local_0_start);
ptrdiff_t fftw_mpi_local_size_many(int rnk, const ptrdiff_t* n, ptrdiff_t howmany, ptrdiff_t block0, MPI_Comm comm,
                                   ptrdiff_t* local_n0, ptrdiff_t* local_0_start);

fftw_plan fftw_mpi_plan_dft_r2c_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, double* in, fftw_complex* out,
                                   MPI_Comm comm, unsigned flags);
fftw_plan fftw_mpi_plan_dft_c2r_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, fftw_complex* in, double* out,
                                   MPI_Comm comm, unsigned flags);
fftw_plan fftw_mpi_plan_many_dft_r2c(int rnk, const ptrdiff_t* n, ptrdiff_t howmany, ptrdiff_t iblock,
                                     ptrdiff_t oblock, double* in, fftw_complex* out, MPI_Comm comm, unsigned flags);
fftw_plan fftw_mpi_plan_many_dft_c2r(int rnk, const ptrdiff_t* n, ptrdiff_t howmany, ptrdiff_t iblock,
                                     ptrdiff_t oblock, fftw_complex* in, double* out, MPI_Comm comm, unsigned flags);
void fftw_mpi_execute_dft_r2c(const fftw_plan p, double* in, fftw_complex* out);
void fftw_mpi_execute_dft_c2r(const fftw_plan p, fftw_complex* in, double* out);

/* Shim-only: how many plans had the D1 size substitution applied (see
   ref_shim.c), so a test can assert that the hot-path plans took it. */
int ns3d_ref_shim_d1_substitutions(void);
#endif
