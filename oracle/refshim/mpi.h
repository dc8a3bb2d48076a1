/* Single-process stand-in for the few MPI calls that the reference mpk2
 * and pdmpk prep code makes (mpk2/comm_data.c:55-63,
 * mpk2/mpi2_mpkwrtbufs.c:162-180; pdmpk compiles against the exec calls,
 * which this oracle never runs: they return an error).
 * Used only to compile the reference as a test oracle: the rank comes
 * from the MPK_RANK environment variable, MPI is reported as not
 * initialised so the world-size assertion is skipped. */
#ifndef ORACLE_REFSHIM_MPI_H
#define ORACLE_REFSHIM_MPI_H
#include <stdlib.h>
#include <time.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef struct { int s; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_LONG 3
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Initialized(int *flag) { *flag = 0; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) {
  (void)c; const char *e = getenv("MPK_RANK"); *r = e ? atoi(e) : 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) {
  (void)c; const char *e = getenv("MPK_NPART"); *s = e ? atoi(e) : 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Alltoallv(const void *s, const int *sc, const int *sd, MPI_Datatype st, void *r,
                                const int *rc, const int *rd, MPI_Datatype rt, MPI_Comm c) {
  (void)s; (void)sc; (void)sd; (void)st; (void)r; (void)rc; (void)rd; (void)rt; (void)c; return 1; }
static inline int MPI_Ialltoallv(const void *s, const int *sc, const int *sd, MPI_Datatype st, void *r,
                                 const int *rc, const int *rd, MPI_Datatype rt, MPI_Comm c, MPI_Request *q) {
  (void)s; (void)sc; (void)sd; (void)st; (void)r; (void)rc; (void)rd; (void)rt; (void)c; (void)q; return 1; }
static inline int MPI_Wait(MPI_Request *q, MPI_Status *st) { (void)q; (void)st; return 0; }
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int g, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)d; (void)g; (void)c; return 1; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int g, MPI_Comm c, MPI_Status *st) {
  (void)b; (void)n; (void)t; (void)s; (void)g; (void)c; (void)st; return 1; }
static inline double MPI_Wtime(void) {
  struct timespec t; clock_gettime(CLOCK_MONOTONIC, &t); return t.tv_sec + 1e-9 * t.tv_nsec; }
#endif
