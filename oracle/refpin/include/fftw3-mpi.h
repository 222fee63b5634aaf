/* Stand-in for the FFTW3 / FFTW3-MPI interface the reference's sources call
 * (test infrastructure for the oracle's parity pin; not part of the product).
 *
 * One rank owns the whole grid.  Plans are 3D real-to-complex transforms of an
 * n0 x n1 x n2 real array whose rows are padded to 2 (n2/2 + 1) doubles, with
 * FFTW_MPI_TRANSPOSED_OUT (complex output [n1][n0][n2/2 + 1]), and their
 * complex-to-real inverses with FFTW_MPI_TRANSPOSED_IN.  Both are unnormalised
 * discrete Fourier transforms (forward sign -1).  The complex-to-real
 * transform takes the multi-dimensional FFTW data flow: complex inverse DFTs
 * along the two slow axes, then a real inverse along the last axis that reads
 * only the real parts of its kx = 0 and kx = n2/2 entries.  It leaves its
 * input unchanged (FFTW may overwrite it; the reference never reads it after
 * such a transform). */
#ifndef PHAFD_REFPIN_FFTW3_MPI_H
#define PHAFD_REFPIN_FFTW3_MPI_H

#include <stddef.h>
#include "mpi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct refpin_plan* fftw_plan;

#define FFTW_MEASURE 0u
#define FFTW_ESTIMATE (1u << 6)
#define FFTW_MPI_TRANSPOSED_IN (1u << 29)
#define FFTW_MPI_TRANSPOSED_OUT (1u << 30)

void fftw_mpi_init(void);
void fftw_mpi_cleanup(void);
ptrdiff_t fftw_mpi_local_size_3d_transposed(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, MPI_Comm comm,
                                            ptrdiff_t* local_n0, ptrdiff_t* local_0_start, ptrdiff_t* local_n1,
                                            ptrdiff_t* local_1_start);
fftw_plan fftw_mpi_plan_dft_r2c_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, double* in, fftw_complex* out,
                                   MPI_Comm comm, unsigned flags);
fftw_plan fftw_mpi_plan_dft_c2r_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, fftw_complex* in, double* out,
                                   MPI_Comm comm, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
void* fftw_malloc(size_t n);
void fftw_free(void* p);

#ifdef __cplusplus
}
#endif

#endif
