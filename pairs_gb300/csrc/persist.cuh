// Grid-wide barriers and cooperative launches for the persistent time-step kernels
// (persist.cu: one system; ensemble.cu: a batched ensemble).
#pragma once

#include "common.cuh"

namespace pg {

constexpr int kBarrierTimeout = 16;          // status->overflow bit: a grid barrier wait ran out

// header of the caller's workspace (the near-cutoff queue's records follow at 256)
struct PersistWs {
    int32_t *cut_count;                      // +0
    unsigned *arrivals;                      // +64
    unsigned *generation;                    // +128
    int32_t *abort;                          // +192
    int2 *records;                           // +256
    int capacity;
};

__host__ __device__ inline PersistWs persist_ws(void *base, int64_t bytes) {
    char *b = reinterpret_cast<char *>(base);
    PersistWs w;
    w.cut_count = reinterpret_cast<int32_t *>(b);
    w.arrivals = reinterpret_cast<unsigned *>(b + 64);
    w.generation = reinterpret_cast<unsigned *>(b + 128);
    w.abort = reinterpret_cast<int32_t *>(b + 192);
    w.records = reinterpret_cast<int2 *>(b + 256);
    const int64_t cap = (bytes - 256) / 8;
    w.capacity = (int) (cap < INT32_MAX ? cap : INT32_MAX);
    return w;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier for a cooperative launch of `nblocks` blocks expecting `expected`
// arrivals.  Returns false when the launch must stop (this or another block's wait ran
// out); never waits longer than limit_ns.
static __device__ bool grid_barrier(const PersistWs &w, unsigned expected, unsigned long long limit_ns, pg_status *status) {
    __shared__ int s_go;
    __syncthreads();
    if(threadIdx.x == 0) {
        int go = 1;
        volatile unsigned *gen = w.generation;
        volatile int32_t *abort = w.abort;
        const unsigned g = *gen;
        __threadfence();                                     // release this block's writes
        if(atomicAdd(w.arrivals, 1u) == expected - 1) {
            atomicExch(w.arrivals, 0u);
            __threadfence();
            atomicAdd(w.generation, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            while(*gen == g) {
                if(*abort) { go = 0; break; }
                if(global_ns() - t0 > limit_ns) {
                    atomicExch(w.abort, 1);
                    atomicOr(&status->overflow, kBarrierTimeout);
                    go = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        s_go = go && *abort == 0;
    }
    __syncthreads();
    __threadfence();                                         // acquire the other blocks' writes
    return s_go != 0;
}

// Blocks of a cooperative launch for kernel slot `slot` (see persist.cu).
int cooperative_grid(int slot, const void *kernel, int block, int *grid);

inline unsigned long long timeout_ns(double seconds) {
    return (unsigned long long) ((seconds > 0.0 ? seconds : 2.0) * 1e9);
}

}  // namespace pg
