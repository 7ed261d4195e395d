/*
 * TEST INFRASTRUCTURE ONLY. Implementations behind oracle/shim/*.h: a single
 * MPI rank, an FFTW 2 MPI plan that runs the oracle's complex FFT, and the GSL
 * mt19937 / uniform / polar-Gaussian conventions from the oracle.
 */
#include <stdlib.h>
#include <string.h>
#include "mpi.h"
#include "fftw_mpi.h"
#include "gsl/gsl_rng.h"
#include "gsl/gsl_randist.h"
#include "../stz_oracle.h"

/* ---- MPI, one rank ---- */
int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_size(MPI_Comm c, int* size) { (void)c; *size = 1; return 0; }
int MPI_Comm_rank(MPI_Comm c, int* rank) { (void)c; *rank = 0; return 0; }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static size_t type_size(MPI_Datatype t) { return t == MPI_INT ? sizeof(int) : t == MPI_FLOAT ? sizeof(float) : sizeof(double); }
int MPI_Allreduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
  (void)op; (void)c;
  memmove(out, in, type_size(t) * (size_t)n);
  return 0;
}
/* With one rank the reference still posts a send to rank 1 from KMC's
 * prefix chain (evolution.c:154-156); there is no receiver, so it is dropped. */
int MPI_Send(const void* b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return 0;
}
int MPI_Recv(void* b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status* st) {
  (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; abort();
}
int MPI_Abort(MPI_Comm c, int code) { (void)c; exit(code == 0 ? 1 : (code & 0xff)); }
int MPI_File_open(MPI_Comm c, const char* name, int mode, MPI_Info info, MPI_File* fh) {
  (void)c; (void)mode; (void)info;
  *fh = fopen(name, "wb");
  return *fh ? 0 : 1;
}
int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype et, MPI_Datatype ft, const char* rep, MPI_Info info) {
  (void)et; (void)ft; (void)rep; (void)info;
  return fseek(fh, (long)disp, SEEK_SET);
}
int MPI_File_write(MPI_File fh, const void* buf, int n, MPI_Datatype t, MPI_Status* st) {
  (void)st;
  return fwrite(buf, type_size(t), (size_t)n, fh) == (size_t)n ? 0 : 1;
}
int MPI_File_close(MPI_File* fh) { fclose(*fh); *fh = NULL; return 0; }

/* ---- FFTW 2 MPI ---- */
struct stz_shim_plan { int nx, ny, sign; };
fftwnd_mpi_plan fftw2d_mpi_create_plan(MPI_Comm comm, int nx, int ny, fftw_direction dir, int flags) {
  (void)comm; (void)flags;
  fftwnd_mpi_plan p = (fftwnd_mpi_plan)malloc(sizeof(*p));
  p->nx = nx; p->ny = ny; p->sign = (int)dir;
  return p;
}
void fftwnd_mpi_local_sizes(fftwnd_mpi_plan p, int* lnx, int* lxs, int* lny, int* lys, int* total) {
  *lnx = p->nx; *lxs = 0; *lny = p->ny; *lys = 0; *total = p->nx * p->ny;
}
void fftwnd_mpi(fftwnd_mpi_plan p, int n_fields, fftw_complex* data, fftw_complex* work, fftwnd_mpi_output_order o) {
  (void)n_fields; (void)work; (void)o;
  or_fft3(1, p->nx, p->ny, (double*)data, p->sign);
}
void fftwnd_mpi_destroy_plan(fftwnd_mpi_plan p) { free(p); }
void* fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void* p) { free(p); }

/* ---- GSL ---- */
struct gsl_rng { or_rng st; };
static const gsl_rng_type shim_mt19937 = {"mt19937"};
const gsl_rng_type* gsl_rng_default = &shim_mt19937;
unsigned long int gsl_rng_default_seed = 0;
gsl_rng* gsl_rng_alloc(const gsl_rng_type* T) {
  (void)T;
  gsl_rng* r = (gsl_rng*)malloc(sizeof(gsl_rng));
  or_rng_seed(&r->st, gsl_rng_default_seed);
  return r;
}
void gsl_rng_free(gsl_rng* r) { free(r); }
double gsl_rng_uniform(const gsl_rng* r) { return or_rng_uniform((or_rng*)&r->st); }
double gsl_rng_uniform_pos(const gsl_rng* r) { return or_rng_uniform_pos((or_rng*)&r->st); }
double gsl_ran_gaussian(const gsl_rng* r, double sigma) { return or_ran_gaussian((or_rng*)&r->st, sigma); }
