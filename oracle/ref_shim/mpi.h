/* Single-process MPI stand-in for building the reference's correlator-node
 * classes as a CPU checker (test infrastructure only).
 *
 * MPI_Pack copies bytes like a homogeneous MPI would; MPI_Send appends the
 * message to an in-process log that the checker harness reads back (this is
 * how Correlation_core::tsys_write hands its record to the output node,
 * sfxc/src/correlation_core.cc:480-513).
 */
#ifndef SFXC_REF_SHIM_MPI_H
#define SFXC_REF_SHIM_MPI_H
#include <stddef.h>

typedef int MPI_Datatype;
typedef int MPI_Comm;
typedef int MPI_Group;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR, count; } MPI_Status;

#define MPI_CHAR 1
#define MPI_UNSIGNED_CHAR 1
#define MPI_BYTE 1
#define MPI_SHORT 2
#define MPI_UNSIGNED_SHORT 2
#define MPI_INT 4
#define MPI_UNSIGNED 4
#define MPI_FLOAT 5
#define MPI_LONG_LONG 8
#define MPI_LONG 8
#define MPI_UNSIGNED_LONG 8
#define MPI_DOUBLE 9
#define MPI_PACKED 1
#define MPI_COMM_WORLD 0
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_SUCCESS 0
#define MPI_THREAD_MULTIPLE 3

#ifdef __cplusplus
extern "C" {
#endif
int MPI_Pack(const void *inbuf, int incount, MPI_Datatype datatype, void *outbuf,
             int outsize, int *position, MPI_Comm comm);
int MPI_Send(const void *buf, int count, MPI_Datatype datatype, int dest, int tag,
             MPI_Comm comm);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
#ifdef __cplusplus
}
#endif
#endif
