/*
 * phpc_summa.h - SUMMA layer of the drop-in (reference src/phpc_summa.h:6-8).
 *
 * C = C + A * B for N x N row-major host matrices distributed over a 2-D
 * periodic Cartesian communicator: the k dimension is cut into lcm(r, c)
 * panels; at step k the owner column broadcasts its A panel along the process
 * row, the owner row its B panel along the process column, and every process
 * adds A_panel * B_panel into its C block through the local GEMM; the blocks
 * are then gathered on rank 0. The local GEMM is phpc_gemm_cuda (plain FP64)
 * or phpc_gemm_cublas (FP64-accurate Ozaki GEMM).
 *
 * Include <mpi.h> from a real MPI, or include/mpi_shim/mpi.h for the
 * single-rank build used on one-GPU nodes (`mpirun -np 1`).
 */
#ifndef PHPC_SUMMA_H
#define PHPC_SUMMA_H

#include <mpi.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reference: phpc_gemm_summa_cuda, src/phpc_summa.c:124-126. */
void phpc_gemm_summa_cuda(MPI_Comm grid_comm, const double *A, const double *B, double *C, int n, int gpu_count,
                          int grid_width, int grid_height, int block_width, float *compute_time);

/* Reference: phpc_gemm_summa_cublas, src/phpc_summa.c:128-130. */
void phpc_gemm_summa_cublas(MPI_Comm grid_comm, const double *A, const double *B, double *C, int n, int gpu_count,
                            float *compute_time);

/* Status of the last SUMMA call on this thread: 0, a PHPC_ERR_* code of the
 * local GEMM, or 0x100 | MPI error code. (No counterpart in the reference,
 * whose SUMMA functions return nothing.) */
int phpc_summa_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* PHPC_SUMMA_H */
