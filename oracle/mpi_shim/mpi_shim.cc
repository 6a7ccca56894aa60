// Single-rank MPI shim for building the reference multigrid as a CPU oracle.
// Test infrastructure only (see mpi.h).  Messages are self-addressed: a send
// is matched to the oldest posted receive with the same tag, or queued until
// such a receive is posted.  MPI_Abort throws, so a fatal error inside the
// reference library becomes an error code in the oracle harness instead of
// killing the test process.
#include "mpi.h"

#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

struct PendingRecv {
    void *buf;
    size_t bytes;
    int tag;
};

struct QueuedMsg {
    std::vector<char> data;
    int tag;
};

std::deque<PendingRecv> g_recvs;
std::deque<QueuedMsg> g_msgs;
int g_next_comm = 2;
std::map<MPI_Comm, std::vector<int>> g_cart_periods;

size_t type_size(MPI_Datatype t) {
    switch (t) {
        case MPI_BYTE: return 1;
        case MPI_CHAR: return 1;
        case MPI_INT: return sizeof(int);
        case MPI_DOUBLE: return sizeof(double);
        case MPI_FLOAT: return sizeof(float);
        default: throw std::runtime_error("mpi shim: unknown datatype");
    }
}

}  // namespace

extern "C" {

int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }

int MPI_Abort(MPI_Comm, int code) {
    throw std::runtime_error("reference library aborted with code " + std::to_string(code));
}

int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_free(MPI_Comm *comm) { *comm = MPI_COMM_NULL; return MPI_SUCCESS; }

int MPI_Comm_split(MPI_Comm, int color, int, MPI_Comm *newcomm) {
    *newcomm = (color == MPI_UNDEFINED) ? MPI_COMM_NULL : g_next_comm++;
    return MPI_SUCCESS;
}

int MPI_Cart_create(MPI_Comm, int ndims, const int *dims, const int *periods, int, MPI_Comm *cart) {
    for (int d = 0; d < ndims; d++)
        if (dims[d] != 1) throw std::runtime_error("mpi shim: Cartesian grid must be 1x1x1");
    *cart = g_next_comm++;
    std::vector<int> &p = g_cart_periods[*cart];
    p.assign(periods, periods + ndims);
    return MPI_SUCCESS;
}

// One rank: every dimension has extent 1 and coordinate 0.
int MPI_Cart_get(MPI_Comm comm, int maxdims, int *dims, int *periods, int *coords) {
    auto it = g_cart_periods.find(comm);
    for (int d = 0; d < maxdims; d++) {
        dims[d] = 1;
        periods[d] = (it != g_cart_periods.end() && d < (int)it->second.size()) ? it->second[d] : 0;
        coords[d] = 0;
    }
    return MPI_SUCCESS;
}

// The neighbours along a dimension: this rank itself if it is periodic, else none.
int MPI_Cart_shift(MPI_Comm comm, int direction, int, int *source, int *dest) {
    auto it = g_cart_periods.find(comm);
    const bool per = it != g_cart_periods.end() && direction < (int)it->second.size() && it->second[direction];
    *source = *dest = per ? 0 : MPI_PROC_NULL;
    return MPI_SUCCESS;
}

int MPI_Cart_rank(MPI_Comm, const int *, int *rank) { *rank = 0; return MPI_SUCCESS; }

int MPI_Cart_coords(MPI_Comm, int, int maxdims, int *coords) {
    for (int d = 0; d < maxdims; d++) coords[d] = 0;
    return MPI_SUCCESS;
}

int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm,
              MPI_Request *req) {
    if (req) *req = 0;
    if (dest == MPI_PROC_NULL) return MPI_SUCCESS;   // no neighbour (a non-periodic edge): nothing moves
    if (dest != 0) throw std::runtime_error("mpi shim: send to a rank other than 0");
    size_t bytes = (size_t)count * type_size(type);
    if (req) *req = 0;
    for (auto it = g_recvs.begin(); it != g_recvs.end(); ++it) {
        if (it->tag == tag) {
            if (it->bytes != bytes) throw std::runtime_error("mpi shim: message size mismatch");
            if (bytes) std::memcpy(it->buf, buf, bytes);
            g_recvs.erase(it);
            return MPI_SUCCESS;
        }
    }
    QueuedMsg m;
    m.data.assign((const char *)buf, (const char *)buf + bytes);
    m.tag = tag;
    g_msgs.push_back(std::move(m));
    return MPI_SUCCESS;
}

int MPI_Irecv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm,
              MPI_Request *req) {
    if (req) *req = 0;
    if (src == MPI_PROC_NULL) return MPI_SUCCESS;   // no neighbour: the buffer is left as it is
    if (src != 0) throw std::runtime_error("mpi shim: receive from a rank other than 0");
    size_t bytes = (size_t)count * type_size(type);
    if (req) *req = 0;
    for (auto it = g_msgs.begin(); it != g_msgs.end(); ++it) {
        if (it->tag == tag) {
            if (it->data.size() != bytes) throw std::runtime_error("mpi shim: message size mismatch");
            if (bytes) std::memcpy(buf, it->data.data(), bytes);
            g_msgs.erase(it);
            return MPI_SUCCESS;
        }
    }
    g_recvs.push_back(PendingRecv{buf, bytes, tag});
    return MPI_SUCCESS;
}

int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm) {
    return MPI_Isend(buf, count, type, dest, tag, comm, nullptr);
}

int MPI_Recv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm,
             MPI_Status *) {
    if (src == MPI_PROC_NULL) return MPI_SUCCESS;
    MPI_Irecv(buf, count, type, src, tag, comm, nullptr);
    if (!g_recvs.empty() && g_recvs.back().buf == buf)
        throw std::runtime_error("mpi shim: blocking receive with no matching send");
    return MPI_SUCCESS;
}

int MPI_Wait(MPI_Request *, MPI_Status *) {
    if (!g_recvs.empty()) throw std::runtime_error("mpi shim: wait on an unmatched receive");
    return MPI_SUCCESS;
}

int MPI_Waitall(int, MPI_Request *, MPI_Status *) {
    // Every send was matched or queued eagerly.  A receive still pending here
    // would deadlock a real MPI run; report it instead.
    if (!g_recvs.empty()) throw std::runtime_error("mpi shim: waitall with unmatched receives");
    return MPI_SUCCESS;
}

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op,
                  MPI_Comm) {
    if (sendbuf != recvbuf) std::memcpy(recvbuf, sendbuf, (size_t)count * type_size(type));
    return MPI_SUCCESS;
}

int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op,
               int, MPI_Comm) {
    if (sendbuf != recvbuf) std::memcpy(recvbuf, sendbuf, (size_t)count * type_size(type));
    return MPI_SUCCESS;
}

int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

double MPI_Wtime(void) {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int stz_shim_pending_receives(void) { return (int)g_recvs.size(); }

void stz_shim_reset(void) {
    g_recvs.clear();
    g_msgs.clear();
}

}  // extern "C"
