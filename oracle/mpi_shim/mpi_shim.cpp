// Single-rank implementation of the MPI stand-in declared in mpi.h (oracle build only).
#include "mpi.h"
#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <deque>
#include <vector>
#include <sys/time.h>

namespace {

size_t type_size(MPI_Datatype t) { return (size_t)(t & 0xff); }

struct Message {
    int tag;
    std::vector<char> data;
};

struct PendingRecv {
    int id;
    void* buf;
    size_t capacity;
    int tag;
    bool done;
};

std::deque<Message>& mailbox() { static std::deque<Message> m; return m; }
std::vector<PendingRecv>& pending() { static std::vector<PendingRecv> p; return p; }
int next_request_id() { static int id = 0; return ++id; }

bool take_message(int tag, void* buf, size_t capacity) {
    std::deque<Message>& box = mailbox();
    for (std::deque<Message>::iterator it = box.begin(); it != box.end(); ++it) {
        if (tag == MPI_ANY_TAG || it->tag == tag) {
            size_t n = it->data.size() < capacity ? it->data.size() : capacity;
            if (n) std::memcpy(buf, &it->data[0], n);
            box.erase(it);
            return true;
        }
    }
    return false;
}

void deliver(const void* buf, size_t bytes, int tag) {
    Message m;
    m.tag = tag;
    m.data.assign((const char*)buf, (const char*)buf + bytes);
    mailbox().push_back(m);
    // satisfy posted receives in order
    std::vector<PendingRecv>& p = pending();
    for (size_t i = 0; i < p.size(); ++i) {
        if (!p[i].done && take_message(p[i].tag, p[i].buf, p[i].capacity)) p[i].done = true;
    }
}

template <class V>
void reduce_typed(const void* in, void* out, int count, MPI_Op op) {
    // one rank: every reduction is the identity
    (void)op;
    if (in != out) std::memmove(out, in, count * sizeof(V));
}

}  // namespace

extern "C" {

int MPI_Init(int*, char***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Initialized(int* flag) { *flag = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
double MPI_Wtime(void) {
    struct timeval tv;
    gettimeofday(&tv, 0);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
}
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm, int code) { std::exit(code); return MPI_SUCCESS; }

int MPI_Send(void* buf, int count, MPI_Datatype type, int, int tag, MPI_Comm) {
    deliver(buf, count * type_size(type), tag);
    return MPI_SUCCESS;
}
int MPI_Rsend(void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm) {
    return MPI_Send(buf, count, type, dest, tag, comm);
}
int MPI_Isend(void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request* req) {
    MPI_Send(buf, count, type, dest, tag, comm);
    *req = MPI_REQUEST_NULL;
    return MPI_SUCCESS;
}
int MPI_Irecv(void* buf, int count, MPI_Datatype type, int, int tag, MPI_Comm, MPI_Request* req) {
    PendingRecv r;
    r.id = next_request_id();
    r.buf = buf;
    r.capacity = count * type_size(type);
    r.tag = tag;
    r.done = take_message(tag, buf, r.capacity);
    pending().push_back(r);
    *req = r.id;
    return MPI_SUCCESS;
}
int MPI_Recv(void* buf, int count, MPI_Datatype type, int, int tag, MPI_Comm, MPI_Status* status) {
    if (!take_message(tag, buf, count * type_size(type))) {
        std::fprintf(stderr, "mpi shim: receive with no matching message (tag %d)\n", tag);
        std::abort();
    }
    if (status) { status->MPI_SOURCE = 0; status->MPI_TAG = tag; status->MPI_ERROR = 0; status->count = count; }
    return MPI_SUCCESS;
}
int MPI_Sendrecv(void* sendbuf, int sendcount, MPI_Datatype sendtype, int, int,
                 void* recvbuf, int recvcount, MPI_Datatype recvtype, int, int, MPI_Comm, MPI_Status*) {
    size_t n = sendcount * type_size(sendtype);
    size_t m = recvcount * type_size(recvtype);
    std::memmove(recvbuf, sendbuf, n < m ? n : m);
    return MPI_SUCCESS;
}
int MPI_Wait(MPI_Request* req, MPI_Status* status) { return MPI_Waitall(1, req, status); }
int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status*) {
    std::vector<PendingRecv>& p = pending();
    for (int i = 0; i < count; ++i) {
        if (reqs[i] == MPI_REQUEST_NULL) continue;
        for (size_t k = 0; k < p.size(); ++k) {
            if (p[k].id != reqs[i]) continue;
            if (!p[k].done && !take_message(p[k].tag, p[k].buf, p[k].capacity)) {
                std::fprintf(stderr, "mpi shim: wait on a receive that can never complete (tag %d)\n", p[k].tag);
                std::abort();
            }
            p.erase(p.begin() + k);
            break;
        }
        reqs[i] = MPI_REQUEST_NULL;
    }
    return MPI_SUCCESS;
}
int MPI_Request_free(MPI_Request* req) { *req = MPI_REQUEST_NULL; return MPI_SUCCESS; }
int MPI_Get_count(MPI_Status* status, MPI_Datatype, int* count) { *count = status ? status->count : 0; return MPI_SUCCESS; }

int MPI_Reduce(void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op, int, MPI_Comm) {
    std::memmove(recvbuf, sendbuf, count * type_size(type));
    (void)op;
    return MPI_SUCCESS;
}
int MPI_Allreduce(void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm) {
    return MPI_Reduce(sendbuf, recvbuf, count, type, op, 0, comm);
}
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
int MPI_Scatterv(void* sendbuf, int* sendcounts, int* displs, MPI_Datatype sendtype,
                 void* recvbuf, int recvcount, MPI_Datatype recvtype, int, MPI_Comm) {
    size_t es = type_size(sendtype);
    size_t n = sendcounts[0] * es, m = recvcount * type_size(recvtype);
    std::memmove(recvbuf, (char*)sendbuf + displs[0] * es, n < m ? n : m);
    return MPI_SUCCESS;
}
int MPI_Gatherv(void* sendbuf, int sendcount, MPI_Datatype sendtype,
                void* recvbuf, int* recvcounts, int* displs, MPI_Datatype recvtype, int, MPI_Comm) {
    size_t er = type_size(recvtype);
    size_t n = sendcount * type_size(sendtype), m = recvcounts[0] * er;
    std::memmove((char*)recvbuf + displs[0] * er, sendbuf, n < m ? n : m);
    return MPI_SUCCESS;
}

int MPI_File_open(MPI_Comm, char*, int, MPI_Info, MPI_File* fh) { *fh = 0; return MPI_ERR_OTHER; }
int MPI_File_close(MPI_File* fh) { *fh = 0; return MPI_ERR_OTHER; }
int MPI_File_seek(MPI_File, MPI_Offset, int) { return MPI_ERR_OTHER; }
int MPI_File_write(MPI_File, void*, int, MPI_Datatype, MPI_Status*) { return MPI_ERR_OTHER; }
int MPI_File_read(MPI_File, void*, int, MPI_Datatype, MPI_Status*) { return MPI_ERR_OTHER; }

}  // extern "C"
