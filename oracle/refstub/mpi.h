/*
 * Single-rank stand-in for the handful of MPI calls made by the reference's
 * .cz writer and reader (SerializerIO_WaveletCompression_MPI_Simple.h:347-466,
 * 468-487, 561-620; Reader_WaveletCompression.h). TEST INFRASTRUCTURE ONLY:
 * it lets the unmodified reference headers compile into oracle/_ref without
 * an MPI installation. Rank 0 of 1; collectives are copies; MPI-IO is POSIX.
 */
#ifndef CZ_REFSTUB_MPI_H
#define CZ_REFSTUB_MPI_H

#include <fcntl.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <unistd.h>

typedef int MPI_Comm;
typedef int MPI_Info;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int fd; long long pos; } *MPI_File;
typedef struct { int dummy; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_COMM_SELF 1
#define MPI_INFO_NULL 0
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_FLOAT 40
#define MPI_UINT64_T 8
#define MPI_LONG 80
#define MPI_DOUBLE 88
#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3
#define MPI_MODE_WRONLY 1
#define MPI_MODE_CREATE 2
#define MPI_MODE_RDONLY 4
#define MPI_THREAD_MULTIPLE 3
#define MPI_IN_PLACE ((void *)1)

static inline int cz_mpi_tsize(MPI_Datatype t)
{
    switch (t) {
    case MPI_CHAR: return 1;
    case MPI_INT: case MPI_FLOAT: return 4;
    default: return 8;
    }
}

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Init_thread(int *, char ***, int, int *p) { if (p) *p = MPI_THREAD_MULTIPLE; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Abort(MPI_Comm, int code) { exit(code); return 0; }
static inline double MPI_Wtime(void)
{
    struct timeval t;
    gettimeofday(&t, 0);
    return t.tv_sec + 1e-6 * t.tv_usec;
}
static inline int MPI_Info_create(MPI_Info *i) { *i = 0; return 0; }
static inline int MPI_Info_set(MPI_Info, char *, char *) { return 0; }
static inline int MPI_Info_free(MPI_Info *) { return 0; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Exscan(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm) { return 0; }
static inline int MPI_Reduce(const void *in, void *out, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
    if (in != MPI_IN_PLACE && in != out) memmove(out, in, (size_t)n * cz_mpi_tsize(t));
    return 0;
}
static inline int MPI_File_open(MPI_Comm, const char *name, int, MPI_Info, MPI_File *f)
{
    *f = (MPI_File)calloc(1, sizeof(**f));
    (*f)->fd = open(name, O_WRONLY | O_CREAT, 0644);
    return (*f)->fd < 0;
}
static inline int MPI_File_write_at(MPI_File f, long long off, const void *buf, int n, MPI_Datatype t, MPI_Status *)
{
    const size_t bytes = (size_t)n * cz_mpi_tsize(t);
    return pwrite(f->fd, buf, bytes, off) != (ssize_t)bytes;
}
static inline int MPI_File_write_at_all(MPI_File f, long long off, const void *buf, int n, MPI_Datatype t, MPI_Status *s)
{
    return MPI_File_write_at(f, off, buf, n, t, s);
}
static inline int MPI_File_write(MPI_File f, const void *buf, int n, MPI_Datatype t, MPI_Status *s)
{
    const int rc = MPI_File_write_at(f, f->pos, buf, n, t, s);
    f->pos += (long long)n * cz_mpi_tsize(t);
    return rc;
}
static inline int MPI_File_close(MPI_File *f)
{
    close((*f)->fd);
    free(*f);
    *f = 0;
    return 0;
}

#endif
