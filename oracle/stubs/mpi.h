/* Single-rank stand-in for the MPI API, used only to compile the reference
 * sources into the pinning library under oracle/_ref (no MPI exists in this
 * image).  Collectives degenerate to copies because there is one rank.
 * Test infrastructure: never linked into the product library. */
#ifndef ORACLE_STUB_MPI_H
#define ORACLE_STUB_MPI_H
#include <string.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;   /* value = size of one element in bytes */
typedef int MPI_Op;
typedef int MPI_Info;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_SUM 0
#define MPI_INFO_NULL 0
#define MPI_THREAD_FUNNELED 1
#define MPI_THREAD_MULTIPLE 3
static inline int MPI_Init_thread(int *a, char ***b, int req, int *prov) { (void)a; (void)b; *prov = req; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c) { (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c)
{ (void)op; (void)root; (void)c; if (s != r) memmove(r, s, (size_t)n * (size_t)t); return 0; }
static inline int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, int root, MPI_Comm c)
{ (void)rn; (void)rt; (void)root; (void)c; memmove(r, s, (size_t)sn * (size_t)st); return 0; }
static inline int MPI_Info_create(MPI_Info *i) { *i = 0; return 0; }
static inline int MPI_Info_set(MPI_Info i, const char *k, const char *v) { (void)i; (void)k; (void)v; return 0; }
static inline int MPI_Info_free(MPI_Info *i) { (void)i; return 0; }
#endif
