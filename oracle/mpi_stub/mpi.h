/*
 * Single-rank stand-in for <mpi.h>, used only to compile the reference's kernel
 * files into oracle/_ref (test infrastructure, never shipped).
 *
 * The reference kernels include EW.h -> Sarray.h -> Require.h, and Require.h
 * (src/Require.h:40, :69-92) pulls in <mpi.h> for its abort macros.  The kernel
 * bodies themselves make no MPI calls; the only symbols the macros touch are
 * MPI_Comm_rank and MPI_Abort, so this header declares just enough types for
 * EW.h to parse and gives those two calls single-rank meanings.
 */
#ifndef SW4G_ORACLE_MPI_STUB_H
#define SW4G_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Info;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_FLOAT 2
#define MPI_INT 3

static inline int MPI_Comm_rank(MPI_Comm comm, int* rank)
{
   (void)comm;
   *rank = 0;
   return 0;
}

static inline int MPI_Abort(MPI_Comm comm, int code)
{
   (void)comm;
   fprintf(stderr, "reference kernel aborted (code %d)\n", code);
   abort();
   return code;
}

#endif
