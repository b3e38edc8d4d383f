/*
 * Single-rank stand-in for <mpi.h>, used only to compile the reference
 * backend's own C sources (libcirc/innerprod.c, libcirc/probability.c,
 * libcirc/utils/comms.c) into the test oracle under oracle/_ref/.
 *
 * With one rank every master/worker loop in the reference degenerates to the
 * master doing all samples itself (libcirc/innerprod.c:69-81 with
 * world_size == 1), so Send/Recv are never reached; they abort if they are.
 *
 * Test infrastructure only: nothing in the product links this header.
 */
#ifndef CSIM_ORACLE_MPI_STUB_H
#define CSIM_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int unused; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *size) { (void)c; *size = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *rank) { (void)c; *rank = 0; return 0; }

static inline int MPI_Send(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm c) {
    (void)buf; (void)count; (void)t; (void)dest; (void)tag; (void)c;
    fprintf(stderr, "mpi stub: MPI_Send reached with one rank\n");
    abort();
}

static inline int MPI_Recv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *st) {
    (void)buf; (void)count; (void)t; (void)src; (void)tag; (void)c; (void)st;
    fprintf(stderr, "mpi stub: MPI_Recv reached with one rank\n");
    abort();
}

#endif
