/* One-rank MPI stand-in for link checks of a C driver written against MPI (the
 * reference's src/main.c): rank 0 of 1, reductions copy, point-to-point calls
 * are no-ops.  Used by tests/test_reference_link_cpu.py only. */
#ifndef MPI_STUB_H
#define MPI_STUB_H
#include <string.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int unused; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_FLOAT 1
#define MPI_SUM 2
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op o, int root, MPI_Comm c)
{ (void)t; (void)o; (void)root; (void)c; memmove(r, s, (size_t)n * sizeof(float)); return 0; }
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return 0; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; return 0; }
static inline int MPI_Finalize(void) { return 0; }
#endif
