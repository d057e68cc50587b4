// simt_shim.h -- run CUDA C++ kernel source on the CPU, one block at a time.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle).  It lets the reference's own
// kernel source (label_propagation/src/dpp/kernel.cuh and
// src/common/segmented_reduce.cuh) be compiled by g++ and executed here, so
// that the CPU restatement in oracle/lp_oracle.c can be pinned against the
// reference itself rather than against a re-derivation.
//
// Model: every CUDA thread of a block is a ucontext fiber on one OS thread.
// A fiber runs until it reaches a synchronisation point (__syncthreads or
// __ballot_sync) and then yields to the scheduler.  When every live fiber has
// yielded, pending ballots are resolved per warp (over the lanes that reached a
// ballot in this round; lanes that did not contribute 0 bits), and otherwise a
// block barrier is released once every live fiber waits at it.  Shared memory
// (`__shared__`) becomes function-static storage, which is correct because
// blocks run one after another.  Atomics are plain read-modify-writes: only
// one fiber runs at any instant.
#pragma once

#include <ucontext.h>
#include <sys/types.h>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <functional>
#include <iterator>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __inline__ inline
#define __forceinline__ inline
#define __shared__ static
#define __restrict__

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

namespace simt {

enum State { READY, AT_BARRIER, AT_BALLOT, DONE };

struct Fiber {
    ucontext_t ctx;
    State st;
    int pred;
    unsigned result;
};

struct Engine {
    dim3 thread_idx, block_idx, block_dim, grid_dim;
    std::vector<Fiber> fibers;
    std::vector<char> stacks;
    ucontext_t sched;
    int cur = -1;
    bool flat = false;
    std::function<void()> body;
    static constexpr size_t kStack = 64 * 1024;
};

inline Engine &eng()
{
    static Engine e;
    return e;
}

inline void yield_as(State s)
{
    Engine &E = eng();
    if (E.flat) {
        std::fprintf(stderr, "simt: synchronisation inside a kernel launched flat\n");
        std::abort();
    }
    Fiber &f = E.fibers[E.cur];
    f.st = s;
    swapcontext(&f.ctx, &E.sched);
}

inline void syncthreads() { yield_as(AT_BARRIER); }

inline unsigned ballot(int pred)
{
    Engine &E = eng();
    E.fibers[E.cur].pred = pred != 0;
    yield_as(AT_BALLOT);
    return E.fibers[E.cur].result;
}

inline void fiber_entry()
{
    Engine &E = eng();
    E.body();
    E.fibers[E.cur].st = DONE;
}

// Launch a kernel whose threads synchronise.
template <class F>
void launch(dim3 grid, dim3 block, F &&f)
{
    Engine &E = eng();
    const int T = (int)block.x;
    E.grid_dim = grid;
    E.block_dim = block;
    E.flat = false;
    E.body = [&]() { f(); };
    if ((int)E.fibers.size() < T) {
        E.fibers.resize(T);
        E.stacks.assign((size_t)T * Engine::kStack, 0);
    }
    for (unsigned bx = 0; bx < grid.x; ++bx) {
        E.block_idx = dim3(bx, 0, 0);
        for (int t = 0; t < T; ++t) {
            Fiber &fb = E.fibers[t];
            getcontext(&fb.ctx);
            fb.ctx.uc_stack.ss_sp = &E.stacks[(size_t)t * Engine::kStack];
            fb.ctx.uc_stack.ss_size = Engine::kStack;
            fb.ctx.uc_link = &E.sched;
            makecontext(&fb.ctx, (void (*)())fiber_entry, 0);
            fb.st = READY;
        }
        for (;;) {
            for (int t = 0; t < T; ++t) {
                if (E.fibers[t].st != READY) continue;
                E.cur = t;
                E.thread_idx = dim3((unsigned)t, 0, 0);
                swapcontext(&E.sched, &E.fibers[t].ctx);
            }
            bool any_ballot = false, any_barrier = false;
            for (int t = 0; t < T; ++t) {
                any_ballot |= E.fibers[t].st == AT_BALLOT;
                any_barrier |= E.fibers[t].st == AT_BARRIER;
            }
            if (any_ballot) {
                for (int w = 0; w < (T + 31) / 32; ++w) {
                    unsigned bits = 0;
                    for (int l = 0; l < 32 && w * 32 + l < T; ++l) {
                        const Fiber &fb = E.fibers[w * 32 + l];
                        if (fb.st == AT_BALLOT && fb.pred) bits |= 1u << l;
                    }
                    for (int l = 0; l < 32 && w * 32 + l < T; ++l) {
                        Fiber &fb = E.fibers[w * 32 + l];
                        if (fb.st == AT_BALLOT) {
                            fb.result = bits;
                            fb.st = READY;
                        }
                    }
                }
            } else if (any_barrier) {
                for (int t = 0; t < T; ++t)
                    if (E.fibers[t].st == AT_BARRIER) E.fibers[t].st = READY;
            } else {
                break;
            }
        }
    }
    E.cur = -1;
}

// Launch a kernel that never synchronises: threads run to completion in order.
template <class F>
void launch_flat(dim3 grid, dim3 block, F &&f)
{
    Engine &E = eng();
    E.grid_dim = grid;
    E.block_dim = block;
    E.flat = true;
    for (unsigned bx = 0; bx < grid.x; ++bx) {
        E.block_idx = dim3(bx, 0, 0);
        for (unsigned t = 0; t < block.x; ++t) {
            E.thread_idx = dim3(t, 0, 0);
            f();
        }
    }
    E.flat = false;
}

inline int clz(unsigned x) { return x ? __builtin_clz(x) : 32; }

}  // namespace simt

#define threadIdx (simt::eng().thread_idx)
#define blockIdx (simt::eng().block_idx)
#define blockDim (simt::eng().block_dim)
#define gridDim (simt::eng().grid_dim)

inline void __syncthreads() { simt::syncthreads(); }
inline unsigned __ballot_sync(unsigned, int pred) { return simt::ballot(pred); }
inline int __clz(unsigned x) { return simt::clz(x); }
inline int __clz(int x) { return simt::clz((unsigned)x); }
inline int atomicAdd(int *p, int v)
{
    int old = *p;
    *p = old + v;
    return old;
}
template <class T>
inline T min(T a, T b)
{
    return b < a ? b : a;
}

// Host-side CUDA runtime calls that the reference's host headers make
// (graph.h pins its arrays; outofcore.cuh copies batches).  Host memory only.
typedef int cudaError_t;
typedef void *cudaStream_t;
enum { cudaSuccess = 0 };
enum { cudaHostRegisterDefault = 0, cudaHostRegisterPortable = 1, cudaHostRegisterMapped = 2 };
enum cudaMemcpyKind { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2 };
inline cudaError_t cudaHostRegister(void *, size_t, unsigned) { return cudaSuccess; }
inline cudaError_t cudaHostUnregister(void *) { return cudaSuccess; }
inline cudaError_t cudaMemcpyAsync(void *dst, const void *src, size_t n, cudaMemcpyKind,
                                   cudaStream_t = nullptr)
{
    std::memmove(dst, src, n);
    return cudaSuccess;
}
