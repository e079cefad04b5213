/* mpi.h — a single-process stand-in for the 14 MPI calls of the reference's grid generator
 * (SCU-benchmark/swept-compression-ramp.c), so that the unmodified C program compiles here
 * and its OCFD3d-Mesh.dat can pin the generator restated in flame3d_mhd_gb300/meshgen.py.
 *
 * TEST INFRASTRUCTURE ONLY (oracle/): nothing in the library links it.
 *
 * The ranks of an N-process run execute one after another as separate processes: the rank
 * and size come from F3D_MPI_RANK / F3D_MPI_SIZE (default 0 and 1). The program's ranks
 * exchange nothing but two broadcasts of the parameters read by rank 0 (and, with its
 * Tecplot 3-D output switched on, the slabs of grid.dat, which this stand-in refuses):
 * rank 0 stores each broadcast buffer in mpi_bcast_<n>.bin in the working directory and the
 * later ranks read it back. MPI_File_* map to stdio on a file that is created if missing
 * and never truncated, so each rank writes its slabs at its own offsets into one file as
 * MPI-IO would. Barriers are no-ops. */
#ifndef F3D_MPI_STUB_H
#define F3D_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef FILE* MPI_File;
typedef struct {
    int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_INFO_NULL 0
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1
#define MPI_SEEK_SET SEEK_SET
#define MPI_SEEK_CUR SEEK_CUR
#define MPI_SUCCESS 0

static int f3d_mpi_env(const char* name, int dflt) {
    const char* v = getenv(name);
    return v ? atoi(v) : dflt;
}

static size_t f3d_mpi_size_of(MPI_Datatype t) { return t == MPI_DOUBLE ? sizeof(double) : sizeof(int); }

static int f3d_mpi_bcast_seq = 0;

static inline int MPI_Init(int* argc, char*** argv) {
    (void)argc;
    (void)argv;
    return MPI_SUCCESS;
}
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm c, int* r) {
    (void)c;
    *r = f3d_mpi_env("F3D_MPI_RANK", 0);
    return MPI_SUCCESS;
}
static inline int MPI_Comm_size(MPI_Comm c, int* s) {
    (void)c;
    *s = f3d_mpi_env("F3D_MPI_SIZE", 1);
    return MPI_SUCCESS;
}
static inline int MPI_Barrier(MPI_Comm c) {
    (void)c;
    return MPI_SUCCESS;
}

static inline int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm c) {
    (void)c;
    char name[64];
    snprintf(name, sizeof(name), "mpi_bcast_%d.bin", f3d_mpi_bcast_seq++);
    const size_t n = (size_t)count * f3d_mpi_size_of(t);
    int rank = f3d_mpi_env("F3D_MPI_RANK", 0);
    FILE* f = fopen(name, rank == root ? "wb" : "rb");
    if (!f || (rank == root ? fwrite(buf, 1, n, f) : fread(buf, 1, n, f)) != n) {
        fprintf(stderr, "mpi stand-in: broadcast %s failed (run rank %d first)\n", name, root);
        exit(2);
    }
    fclose(f);
    return MPI_SUCCESS;
}

static inline int MPI_File_open(MPI_Comm c, const char* name, int mode, MPI_Info info, MPI_File* fh) {
    (void)c;
    (void)mode;
    (void)info;
    *fh = fopen(name, "r+b");
    if (!*fh) *fh = fopen(name, "w+b");
    if (!*fh) {
        fprintf(stderr, "mpi stand-in: cannot open %s\n", name);
        exit(2);
    }
    return MPI_SUCCESS;
}
static inline int MPI_File_seek(MPI_File fh, MPI_Offset off, int whence) {
    return fseek(fh, (long)off, whence) == 0 ? MPI_SUCCESS : 1;
}
static inline int MPI_File_write(MPI_File fh, const void* buf, int count, MPI_Datatype t, MPI_Status* st) {
    (void)st;
    const size_t n = (size_t)count * f3d_mpi_size_of(t);
    return fwrite(buf, 1, n, fh) == n ? MPI_SUCCESS : 1;
}
static inline int MPI_File_close(MPI_File* fh) {
    fclose(*fh);
    *fh = NULL;
    return MPI_SUCCESS;
}

static inline int MPI_Send(const void* b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) {
    (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c;
    fprintf(stderr, "mpi stand-in: point-to-point messages are not supported (Tecplot 3-D output)\n");
    exit(2);
}
static inline int MPI_Recv(void* b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status* st) {
    (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st;
    fprintf(stderr, "mpi stand-in: point-to-point messages are not supported (Tecplot 3-D output)\n");
    exit(2);
}

#endif
