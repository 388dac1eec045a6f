/*
 * Single-rank MPI for building the reference's hot path as a CPU checker.
 * Test infrastructure only: it exists so that dataLL.cpp (which calls MPI in
 * updateDomain, dataLL.cpp:319-700) links without an MPI library.  Point to
 * point messages are loop-backed: a rank that is its own periodic neighbour
 * (misc.cpp:690-716) receives exactly what it sent, matched by tag, which is
 * how the reference wraps particles and ghosts across periodic axes on one
 * rank.  Collectives copy the single contribution.
 */
#ifndef ORACLE_SHIM_MPI_H
#define ORACLE_SHIM_MPI_H
#include <cstdlib>
#include <cstring>
#include <vector>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
struct MPI_Status { int unused; };
#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_BYTE 2
#define MPI_DOUBLE 3
#define MPI_REQUEST_NULL 0

inline size_t oracle_mpi_size(MPI_Datatype t) {
    return t == MPI_INT ? sizeof(int) : t == MPI_DOUBLE ? sizeof(double) : 1;
}
struct OracleMpiMsg { int tag; const void *src; void *dst; size_t bytes; bool is_send; };
inline std::vector<OracleMpiMsg> &oracle_mpi_queue() { static std::vector<OracleMpiMsg> q; return q; }

inline int MPI_Init(int *, char ***) { return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *r) {
    OracleMpiMsg m = {tag, b, 0, n * oracle_mpi_size(t), true};
    oracle_mpi_queue().push_back(m); *r = 1; return 0;
}
inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *r) {
    OracleMpiMsg m = {tag, 0, b, n * oracle_mpi_size(t), false};
    oracle_mpi_queue().push_back(m); *r = 1; return 0;
}
/* Sends are posted before the matching receives complete; all data moves here. */
inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) {
    std::vector<OracleMpiMsg> &q = oracle_mpi_queue();
    for (size_t i = 0; i < q.size(); i++) {
        if (q[i].is_send) continue;
        bool matched = false;
        for (size_t j = 0; j < q.size(); j++) {
            if (q[j].is_send && q[j].tag == q[i].tag && q[j].src) {
                if (q[j].bytes > q[i].bytes) std::abort();
                std::memcpy(q[i].dst, q[j].src, q[j].bytes);
                q[j].src = 0;
                matched = true;
                break;
            }
        }
        if (!matched) std::abort();
    }
    q.clear();
    return 0;
}
inline int MPI_Allgather(const void *a, int n, MPI_Datatype t, void *b, int, MPI_Datatype, MPI_Comm) {
    std::memcpy(b, a, n * oracle_mpi_size(t)); return 0;
}
inline int MPI_Gather(const void *a, int n, MPI_Datatype t, void *b, int, MPI_Datatype, int, MPI_Comm) {
    std::memcpy(b, a, n * oracle_mpi_size(t)); return 0;
}
inline int MPI_Scatter(const void *a, int n, MPI_Datatype t, void *b, int, MPI_Datatype, int, MPI_Comm) {
    std::memcpy(b, a, n * oracle_mpi_size(t)); return 0;
}
#endif
