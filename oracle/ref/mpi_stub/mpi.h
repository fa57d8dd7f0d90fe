// Single-rank stand-in for <mpi.h>, used only to build the reference MPI
// programs (mpi_evolution.cpp, moore_mpi_evolution.cpp) as the oracle's
// reference binaries.  TEST INFRASTRUCTURE ONLY.
//
// With one rank every MPI_Sendrecv in those programs sends to itself, so it is
// a memmove; this is exactly the periodic wrap of the halo planes
// (mpi_evolution.cpp:318-332,925-943).  MPI_Send/MPI_Recv are only reached
// with more than one rank and abort here.
//
// MPI_Finalize() additionally dumps the core of every field vector (both time
// slots, full double precision) to the file named by $AXR_DUMP.  The macro is
// expanded inside the reference's main(), where the names listed in
// AXR_FIELDS (set on the compile line, e.g. totSize,haloSize,coreSize,phi,theta)
// are in scope.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int unused; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

inline int MPI_Init(int*, char***) { return 0; }
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }

inline int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int, int,
                        void* recvbuf, int recvcount, MPI_Datatype recvtype, int, int,
                        MPI_Comm, MPI_Status*)
{
    if ((size_t)sendcount * sendtype != (size_t)recvcount * recvtype) std::abort();
    std::memmove(recvbuf, sendbuf, (size_t)sendcount * (size_t)sendtype);
    return 0;
}

inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { std::abort(); }
inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { std::abort(); }

inline void axr_dump_one(std::FILE* f, int totSize, int haloSize, int coreSize, const std::vector<double>& v)
{
    const size_t nslots = v.size() / (size_t)totSize;  // comps * 2
    for (size_t cs = 0; cs < nslots; ++cs)
        std::fwrite(&v[cs * (size_t)totSize + (size_t)haloSize], sizeof(double), (size_t)coreSize, f);
}

template <class... V>
inline int axr_finalize_dump(int totSize, int haloSize, int coreSize, const V&... vs)
{
    const char* path = std::getenv("AXR_DUMP");
    if (!path) return 0;
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return 1;
    (axr_dump_one(f, totSize, haloSize, coreSize, vs), ...);
    std::fclose(f);
    return 0;
}

#define MPI_Finalize() axr_finalize_dump(AXR_FIELDS)
