/* Project-written single-rank stand-in for the MPI calls kspace-neutrinos makes
 * (powerspectrum.c:91-95, interface_common.c:56-186, interface_gadget.c:189).
 * Allreduce copies (or, when a hook is installed, delegates to the hook so a test
 * harness can emulate several ranks); Bcast and Barrier are no-ops.
 * Test infrastructure: not shipped. */
#ifndef KSP_SHIM_MPI_H
#define KSP_SHIM_MPI_H
#include <string.h>
#include <stdlib.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_LONG_LONG_INT 3
#define MPI_BYTE 4
#define MPI_LONG 5
#define MPI_SUM 1
#define MPI_SUCCESS 0
#define MPI_IN_PLACE ((void *)1)
#ifdef __cplusplus
extern "C" {
#endif
/* Optional hook: sums `count` items of `dt` across emulated ranks in place. */
extern int (*kspace_shim_allreduce_hook)(void *buf, int count, MPI_Datatype dt);
#ifdef __cplusplus
}
#endif
static inline size_t kspace_shim_mpi_size(MPI_Datatype dt)
{
    switch (dt) {
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_LONG_LONG_INT: return sizeof(long long);
    case MPI_LONG: return sizeof(long);
    default: return 1;
    }
}
static inline int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype dt,
                                MPI_Op op, MPI_Comm comm)
{
    (void)op; (void)comm;
    if (sendbuf != MPI_IN_PLACE)
        memcpy(recvbuf, sendbuf, (size_t)count * kspace_shim_mpi_size(dt));
    if (kspace_shim_allreduce_hook)
        return kspace_shim_allreduce_hook(recvbuf, count, dt);
    return 0;
}
static inline int MPI_Bcast(void *buf, int count, MPI_Datatype dt, int root, MPI_Comm comm)
{ (void)buf; (void)count; (void)dt; (void)root; (void)comm; return 0; }
static inline int MPI_Barrier(MPI_Comm comm) { (void)comm; return 0; }
static inline int MPI_Abort(MPI_Comm comm, int code) { (void)comm; exit(code); return 0; }
static inline int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return 0; }
static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
#endif
