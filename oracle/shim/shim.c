/* Implementations behind the stand-in headers in this directory.  They let the
   reference's own 2LPT sources compile as a single process for the oracle
   (test infrastructure only). */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "mpi.h"
#include "drfftw_mpi.h"
#include "gsl/gsl_rng.h"
#include "gsl/gsl_sf_legendre.h"
#include "aar_oracle.h"

static int tsize(MPI_Datatype t) { return t == MPI_INT ? 4 : t == MPI_DOUBLE ? 8 : 1; }
int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
int MPI_Abort(MPI_Comm c, int code) { (void)c; exit(code ? code : 1); }
int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c) { (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
int MPI_Allgather(const void *sb, int sn, MPI_Datatype st, void *rb, int rn, MPI_Datatype rt, MPI_Comm c) {
  (void)rn; (void)rt; (void)c; memcpy(rb, sb, (size_t)sn * tsize(st)); return 0; }
int MPI_Allreduce(const void *sb, void *rb, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
  (void)op; (void)c; memcpy(rb, sb, (size_t)n * tsize(t)); return 0; }
int MPI_Reduce(const void *sb, void *rb, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) {
  (void)op; (void)root; (void)c; memcpy(rb, sb, (size_t)n * tsize(t)); return 0; }
static const void *pending_buf;
static size_t pending_len;
int MPI_Send(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c) {
  (void)dst; (void)tag; (void)c; pending_buf = b; pending_len = (size_t)n * tsize(t); return 0; }
int MPI_Isend(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c, MPI_Request *r) {
  (void)r; return MPI_Send(b, n, t, dst, tag, c); }
int MPI_Recv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *s) {
  (void)src; (void)tag; (void)c; (void)s;
  size_t len = (size_t)n * tsize(t);
  if (pending_buf && len <= pending_len) memmove(b, pending_buf, len);
  pending_buf = NULL;
  return 0; }
int MPI_Wait(MPI_Request *r, MPI_Status *s) { (void)r; (void)s; return 0; }

static gsl_rng_type ranlxd1_type = {202};
const gsl_rng_type *gsl_rng_ranlxd1 = &ranlxd1_type;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *t) {
  gsl_rng *r = (gsl_rng *)calloc(1, sizeof(gsl_rng));
  orc_rlx_seed(&r->s, 0, t->luxury);
  return r; }
void gsl_rng_set(gsl_rng *r, unsigned long seed) { orc_rlx_seed(&r->s, seed, r->s.luxury); }
double gsl_rng_uniform(gsl_rng *r) { return orc_rlx_uniform(&r->s); }
void gsl_rng_free(gsl_rng *r) { free(r); }

double gsl_sf_legendre_Pl(int l, double x) {
  if (l == 0) return 1.0;
  double p0 = 1.0, p1 = x;
  for (int n = 2; n <= l; ++n) { double p2 = ((2 * n - 1) * x * p1 - (n - 1) * p0) / n; p0 = p1; p1 = p2; }
  return p1; }

rfftwnd_mpi_plan rfftw3d_mpi_create_plan(MPI_Comm c, int nx, int ny, int nz, fftw_direction dir, int flags) {
  (void)c; (void)ny; (void)nz; (void)flags;
  rfftwnd_mpi_plan p = (rfftwnd_mpi_plan)malloc(sizeof(*p)); p->n = nx; p->dir = dir; return p; }
void rfftwnd_mpi_local_sizes(rfftwnd_mpi_plan p, int *lnx, int *lx0, int *lny, int *ly0, int *tot) {
  *lnx = p->n; *lx0 = 0; *lny = p->n; *ly0 = 0; *tot = p->n * p->n * 2 * (p->n / 2 + 1); }
void rfftwnd_mpi(rfftwnd_mpi_plan p, int nf, fftw_real *data, fftw_real *work, fftwnd_mpi_output_order o) {
  (void)nf; (void)work; (void)o;
  int N = p->n, H = N / 2 + 1;
  size_t rows = (size_t)N * N;
  double *r = (double *)malloc(sizeof(double) * rows * N);
  if (p->dir == FFTW_COMPLEX_TO_REAL) {
    orc_c2r_3d(N, data, r);               /* complex view [N][N][H] of the buffer */
    for (size_t q = 0; q < rows; ++q) memcpy(data + q * 2 * H, r + q * N, sizeof(double) * N);
  } else {
    for (size_t q = 0; q < rows; ++q) memcpy(r + q * N, data + q * 2 * H, sizeof(double) * N);
    orc_r2c_3d(N, r, data);
  }
  free(r); }
void rfftwnd_mpi_destroy_plan(rfftwnd_mpi_plan p) { free(p); }
