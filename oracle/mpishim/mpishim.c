/*
 * mpishim.c -- fork + shared-memory implementation of the MPI subset that the
 * reference 3dmhd code uses.  Test infrastructure for the parity oracle only.
 * See mpi.h for the contract.
 */
#define _GNU_SOURCE
#include "mpi.h"

#include <errno.h>
#include <sched.h>
#include <signal.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/types.h>
#include <sys/wait.h>
#include <time.h>
#include <unistd.h>

#define SHIM_MAX_NP 128
#define SHIM_NSLOT 8
#define SHIM_MAX_RED 8192
#define SHIM_MAX_REQ 64

typedef struct {
    int state; /* 0 empty, 1 full */
    int tag;
    long seq;
    long bytes;
} slot_hdr;

typedef struct {
    int np;
    long slot_bytes;
    int bar_count;
    int bar_sense;
    long chan_seq[SHIM_MAX_NP * SHIM_MAX_NP];
    double red[SHIM_MAX_NP][SHIM_MAX_RED];
} shim_hdr;

typedef struct {
    int active;
    void* buf;
    long bytes;
    int src;
    int tag;
} recv_req;

static shim_hdr* g_hdr = NULL;
static char* g_slots = NULL;
static int g_rank = 0;
static int g_np = 1;
static int g_default_np = 0;
static int g_local_sense = 0;
static double g_timeout_s = 600.0;
static pid_t g_children[SHIM_MAX_NP];
static pid_t g_parent = 0;
static recv_req g_reqs[SHIM_MAX_REQ];

void mpishim_set_default_np(int np) { g_default_np = np; }

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void shim_fail(const char* what) {
    fprintf(stderr, "[mpishim rank %d] %s\n", g_rank, what);
    fflush(stderr);
    if (g_rank == 0) {
        for (int r = 1; r < g_np; r++)
            if (g_children[r] > 0) kill(g_children[r], SIGKILL);
    }
    _exit(3);
}

/* One bounded-wait tick: yields, checks for dead peers and for the time limit. */
static void wait_tick(double t0, long* spins, const char* site) {
    (*spins)++;
    if ((*spins & 63) == 0) {
        struct timespec ts = {0, 20000};
        nanosleep(&ts, NULL);
    } else {
        sched_yield();
    }
    if ((*spins & 1023) == 0) {
        if (now_s() - t0 > g_timeout_s) shim_fail(site);
        if (g_rank == 0) {
            for (int r = 1; r < g_np; r++) {
                int st = 0;
                if (g_children[r] > 0 && waitpid(g_children[r], &st, WNOHANG) == g_children[r]) {
                    g_children[r] = 0;
                    if (!(WIFEXITED(st) && WEXITSTATUS(st) == 0)) {
                        fprintf(stderr, "[mpishim] rank %d died while rank 0 waited in %s\n", r, site);
                        shim_fail("peer failure");
                    }
                }
            }
        } else if (getppid() != g_parent) {
            shim_fail("rank 0 is gone");
        }
    }
}

static size_t dt_size(MPI_Datatype dt) {
    switch (dt) {
        case MPI_DOUBLE: return sizeof(double);
        case MPI_FLOAT: return sizeof(float);
        case MPI_INT: return sizeof(int);
        default: shim_fail("unsupported datatype"); return 0;
    }
}

static slot_hdr* slot_at(int src, int dst, int k) {
    size_t stride = sizeof(slot_hdr) + (size_t)g_hdr->slot_bytes;
    size_t idx = ((size_t)src * (size_t)g_np + (size_t)dst) * SHIM_NSLOT + (size_t)k;
    return (slot_hdr*)(g_slots + idx * stride);
}

int MPI_Init(int* argc, char*** argv) {
    (void)argc;
    (void)argv;
    const char* s = getenv("MPISHIM_NP");
    g_np = s ? atoi(s) : (g_default_np > 0 ? g_default_np : 1);
    if (g_np < 1 || g_np > SHIM_MAX_NP) shim_fail("MPISHIM_NP out of range");
    long slot_bytes = 1L << 20;
    if ((s = getenv("MPISHIM_SLOT_BYTES"))) slot_bytes = atol(s);
    slot_bytes = (slot_bytes + 63) & ~63L;
    if ((s = getenv("MPISHIM_TIMEOUT_S"))) g_timeout_s = atof(s);

    size_t hdr_bytes = (sizeof(shim_hdr) + 4095) & ~(size_t)4095;
    size_t slot_total = (size_t)g_np * (size_t)g_np * SHIM_NSLOT * (sizeof(slot_hdr) + (size_t)slot_bytes);
    void* mem = mmap(NULL, hdr_bytes + slot_total, PROT_READ | PROT_WRITE,
                     MAP_SHARED | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
    if (mem == MAP_FAILED) shim_fail("mmap of the shared arena failed");
    g_hdr = (shim_hdr*)mem;
    g_slots = (char*)mem + hdr_bytes;
    g_hdr->np = g_np;
    g_hdr->slot_bytes = slot_bytes;
    g_parent = getpid();
    memset(g_children, 0, sizeof(g_children));
    memset(g_reqs, 0, sizeof(g_reqs));

    fflush(NULL);
    for (int r = 1; r < g_np; r++) {
        pid_t pid = fork();
        if (pid < 0) shim_fail("fork failed");
        if (pid == 0) {
            g_rank = r;
            return MPI_SUCCESS;
        }
        g_children[r] = pid;
    }
    g_rank = 0;
    return MPI_SUCCESS;
}

int MPI_Finalize(void) {
    fflush(NULL);
    if (g_rank != 0) return MPI_SUCCESS; /* the child's own exit status is what rank 0 sees */
    int bad = 0;
    double t0 = now_s();
    for (int r = 1; r < g_np; r++) {
        if (g_children[r] <= 0) continue;
        int st = 0;
        for (;;) {
            pid_t got = waitpid(g_children[r], &st, WNOHANG);
            if (got == g_children[r]) break;
            if (got < 0 && errno != EINTR) break;
            if (now_s() - t0 > g_timeout_s) {
                kill(g_children[r], SIGKILL);
                waitpid(g_children[r], &st, 0);
                st = 1 << 8;
                break;
            }
            struct timespec ts = {0, 1000000};
            nanosleep(&ts, NULL);
        }
        if (!(WIFEXITED(st) && WEXITSTATUS(st) == 0)) {
            fprintf(stderr, "[mpishim] rank %d exited abnormally (status 0x%x)\n", r, st);
            bad = 1;
        }
        g_children[r] = 0;
    }
    if (bad) _exit(4);
    return MPI_SUCCESS;
}

int MPI_Comm_rank(MPI_Comm comm, int* rank) {
    (void)comm;
    *rank = g_rank;
    return MPI_SUCCESS;
}

int MPI_Comm_size(MPI_Comm comm, int* size) {
    (void)comm;
    *size = g_np;
    return MPI_SUCCESS;
}

int MPI_Barrier(MPI_Comm comm) {
    (void)comm;
    if (g_np == 1) return MPI_SUCCESS;
    g_local_sense = !g_local_sense;
    if (__atomic_add_fetch(&g_hdr->bar_count, 1, __ATOMIC_ACQ_REL) == g_np) {
        __atomic_store_n(&g_hdr->bar_count, 0, __ATOMIC_RELAXED);
        __atomic_store_n(&g_hdr->bar_sense, g_local_sense, __ATOMIC_RELEASE);
    } else {
        double t0 = now_s();
        long spins = 0;
        while (__atomic_load_n(&g_hdr->bar_sense, __ATOMIC_ACQUIRE) != g_local_sense)
            wait_tick(t0, &spins, "MPI_Barrier");
    }
    return MPI_SUCCESS;
}

static void reduce_into(double* acc, const double* v, int n, MPI_Op op) {
    for (int i = 0; i < n; i++) {
        switch (op) {
            case MPI_MIN: acc[i] = acc[i] < v[i] ? acc[i] : v[i]; break;
            case MPI_MAX: acc[i] = acc[i] > v[i] ? acc[i] : v[i]; break;
            case MPI_SUM: acc[i] = acc[i] + v[i]; break;
            default: shim_fail("unsupported reduction op");
        }
    }
}

int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype dt, MPI_Op op, MPI_Comm comm) {
    (void)comm;
    if (dt != MPI_DOUBLE) shim_fail("Allreduce supports doubles only");
    if (count > SHIM_MAX_RED) shim_fail("Allreduce count too large");
    memcpy(g_hdr->red[g_rank], sendbuf, sizeof(double) * (size_t)count);
    MPI_Barrier(comm);
    /* Every rank folds the contributions in rank order, so all ranks get identical bits. */
    double* out = (double*)recvbuf;
    memcpy(out, g_hdr->red[0], sizeof(double) * (size_t)count);
    for (int r = 1; r < g_np; r++) reduce_into(out, g_hdr->red[r], count, op);
    MPI_Barrier(comm);
    return MPI_SUCCESS;
}

static void post_send(const void* buf, long bytes, int dest, int tag) {
    if (dest < 0 || dest >= g_np) shim_fail("send to an invalid rank");
    if (bytes > g_hdr->slot_bytes) shim_fail("message larger than MPISHIM_SLOT_BYTES");
    long* seqp = &g_hdr->chan_seq[g_rank * SHIM_MAX_NP + dest];
    double t0 = now_s();
    long spins = 0;
    for (;;) {
        for (int k = 0; k < SHIM_NSLOT; k++) {
            slot_hdr* sl = slot_at(g_rank, dest, k);
            if (__atomic_load_n(&sl->state, __ATOMIC_ACQUIRE) == 0) {
                sl->tag = tag;
                sl->bytes = bytes;
                sl->seq = (*seqp)++;
                memcpy((char*)(sl + 1), buf, (size_t)bytes);
                __atomic_store_n(&sl->state, 1, __ATOMIC_RELEASE);
                return;
            }
        }
        wait_tick(t0, &spins, "send (all slots busy)");
    }
}

static void complete_recv(void* buf, long bytes, int src, int tag, MPI_Status* st) {
    if (src < 0 || src >= g_np) shim_fail("receive from an invalid rank");
    double t0 = now_s();
    long spins = 0;
    for (;;) {
        slot_hdr* best = NULL;
        for (int k = 0; k < SHIM_NSLOT; k++) {
            slot_hdr* sl = slot_at(src, g_rank, k);
            if (__atomic_load_n(&sl->state, __ATOMIC_ACQUIRE) == 1 && sl->tag == tag) {
                if (!best || sl->seq < best->seq) best = sl;
            }
        }
        if (best) {
            if (best->bytes > bytes) shim_fail("message truncated");
            memcpy(buf, (char*)(best + 1), (size_t)best->bytes);
            if (st) {
                st->MPI_SOURCE = src;
                st->MPI_TAG = tag;
                st->MPI_ERROR = 0;
            }
            __atomic_store_n(&best->state, 0, __ATOMIC_RELEASE);
            return;
        }
        wait_tick(t0, &spins, "receive");
    }
}

int MPI_Send(const void* buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm comm) {
    (void)comm;
    post_send(buf, (long)count * (long)dt_size(dt), dest, tag);
    return MPI_SUCCESS;
}

int MPI_Recv(void* buf, int count, MPI_Datatype dt, int source, int tag, MPI_Comm comm, MPI_Status* status) {
    (void)comm;
    complete_recv(buf, (long)count * (long)dt_size(dt), source, tag, status);
    return MPI_SUCCESS;
}

int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void* recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status* status) {
    MPI_Send(sendbuf, sendcount, sendtype, dest, sendtag, comm);
    return MPI_Recv(recvbuf, recvcount, recvtype, source, recvtag, comm, status);
}

int MPI_Bcast(void* buf, int count, MPI_Datatype dt, int root, MPI_Comm comm) {
    const int bcast_tag = -7771;
    if (g_rank == root) {
        for (int r = 0; r < g_np; r++)
            if (r != root) MPI_Send(buf, count, dt, r, bcast_tag, comm);
    } else {
        MPI_Recv(buf, count, dt, root, bcast_tag, comm, MPI_STATUS_IGNORE);
    }
    return MPI_SUCCESS;
}

int MPI_Isend(const void* buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm comm, MPI_Request* req) {
    MPI_Send(buf, count, dt, dest, tag, comm);
    *req = MPI_REQUEST_NULL;
    return MPI_SUCCESS;
}

int MPI_Irecv(void* buf, int count, MPI_Datatype dt, int source, int tag, MPI_Comm comm, MPI_Request* req) {
    (void)comm;
    for (int i = 0; i < SHIM_MAX_REQ; i++) {
        if (!g_reqs[i].active) {
            g_reqs[i].active = 1;
            g_reqs[i].buf = buf;
            g_reqs[i].bytes = (long)count * (long)dt_size(dt);
            g_reqs[i].src = source;
            g_reqs[i].tag = tag;
            *req = i;
            return MPI_SUCCESS;
        }
    }
    shim_fail("too many pending receives");
    return 1;
}

int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status* statuses) {
    for (int i = 0; i < count; i++) {
        int r = reqs[i];
        if (r == MPI_REQUEST_NULL) continue;
        if (r < 0 || r >= SHIM_MAX_REQ || !g_reqs[r].active) shim_fail("Waitall on an unknown request");
        complete_recv(g_reqs[r].buf, g_reqs[r].bytes, g_reqs[r].src, g_reqs[r].tag,
                      statuses ? &statuses[i] : NULL);
        g_reqs[r].active = 0;
        reqs[i] = MPI_REQUEST_NULL;
    }
    return MPI_SUCCESS;
}
