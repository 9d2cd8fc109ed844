/* Stand-in for the FFTW 2.1.5 MPI real-transform interface the reference
   calls (rfftw3d_mpi_create_plan, rfftwnd_mpi_local_sizes, rfftwnd_mpi,
   rfftwnd_mpi_destroy_plan).  In-place, padded real layout
   [N][N][2(N/2+1)], natural output order, unnormalised, backed by the
   oracle's FP64 FFT.  Test infrastructure only. */
#ifndef AAR_SHIM_DRFFTW_MPI_H
#define AAR_SHIM_DRFFTW_MPI_H
#include <stdio.h>
#include <mpi.h>
typedef double fftw_real;
typedef struct { fftw_real re, im; } fftw_complex;
typedef enum { FFTW_FORWARD = -1, FFTW_BACKWARD = 1 } fftw_direction;
#define FFTW_REAL_TO_COMPLEX FFTW_FORWARD
#define FFTW_COMPLEX_TO_REAL FFTW_BACKWARD
#define FFTW_ESTIMATE 0
typedef enum { FFTW_NORMAL_ORDER, FFTW_TRANSPOSED_ORDER } fftwnd_mpi_output_order;
typedef struct aar_shim_plan { int n, dir; } *rfftwnd_mpi_plan;
rfftwnd_mpi_plan rfftw3d_mpi_create_plan(MPI_Comm c, int nx, int ny, int nz, fftw_direction dir, int flags);
void rfftwnd_mpi_local_sizes(rfftwnd_mpi_plan p, int *local_nx, int *local_x_start, int *local_ny_after,
                             int *local_y_start_after, int *total_local_size);
void rfftwnd_mpi(rfftwnd_mpi_plan p, int n_fields, fftw_real *local_data, fftw_real *work,
                 fftwnd_mpi_output_order order);
void rfftwnd_mpi_destroy_plan(rfftwnd_mpi_plan p);
#endif
