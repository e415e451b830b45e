/*
 * Declarations-only stand-in for <mpi.h> (TEST INFRASTRUCTURE).
 *
 * source/core/msquery.cpp declares two MPI globals (msquery.cpp:25-26) and
 * uses MPI only in MSQuery::init_index / write_index / read_index / archive
 * (msquery.cpp:200-237), which the MS2 reader path (initialize, extractbatch,
 * readspectrum, pickpeaks) never calls. This header lets that translation
 * unit compile without an MPI installation; every function here fails.
 */
#pragma once

typedef int MPI_Datatype;
typedef int MPI_File;
typedef int MPI_Comm;
typedef int MPI_Info;
typedef struct { int unused; } MPI_Status;

#define MPI_INT 0
#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 2
#define MPI_MODE_RDONLY 4
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_ERR_OTHER 15

static inline int MPI_Type_contiguous(int, MPI_Datatype, MPI_Datatype *) { return MPI_ERR_OTHER; }
static inline int MPI_Type_commit(MPI_Datatype *) { return MPI_ERR_OTHER; }
static inline int MPI_File_open(MPI_Comm, const char *, int, MPI_Info, MPI_File *) { return MPI_ERR_OTHER; }
static inline int MPI_File_close(MPI_File *) { return MPI_ERR_OTHER; }
static inline int MPI_File_read_all(MPI_File, void *, int, MPI_Datatype, MPI_Status *) { return MPI_ERR_OTHER; }
static inline int MPI_File_write_at(MPI_File, long, const void *, int, MPI_Datatype, MPI_Status *)
{
    return MPI_ERR_OTHER;
}
