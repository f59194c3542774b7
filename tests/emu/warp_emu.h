// warp_emu.h -- host emulation of the CUDA features the region LZ4 kernels
// use (cubismz_gb300/csrc/cz_lz4rec.cu), so that their exact source runs on
// the CPU under the CPU test suite (and AddressSanitizer).
//
// One warp is 32 lanes run as ucontext coroutines in one OS thread. Every
// warp-synchronous intrinsic (__syncwarp, shuffles, votes) is a sync point
// where the running lane yields to the next; the kernels meet the same sync
// points in the same order on every lane, so a phase ends when every lane
// has reached it. The lane order of each phase is a seeded random
// permutation, so that same-address stores of one phase land in varying
// orders, as on the GPU. Test infrastructure only.
#pragma once
#include <ucontext.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __noinline__
#define __restrict__
#define __launch_bounds__(...)
#define __align__(n) alignas(n)
using std::max;
using std::min;
typedef int cudaError_t;
typedef void *cudaStream_t;

struct EmuDim3 {
    unsigned x = 1, y = 1, z = 1;
};
inline EmuDim3 threadIdx, blockIdx, gridDim, blockDim;
inline unsigned char *g_emu_smem = nullptr;

struct EmuWarp {
    ucontext_t main, lane[32];
    int cur = 0, pos = 0, ndone = 0;
    int perm[32];
    bool done[32];
    unsigned base = 0, rng = 1;
    uint64_t xch[32];
    std::function<void()> *fn = nullptr;
};
inline EmuWarp g_emu;

inline void emu_perm()
{
    for (int i = 0; i < 32; ++i) g_emu.perm[i] = i;
    for (int i = 31; i > 0; --i) {
        g_emu.rng = g_emu.rng * 1103515245u + 12345u;
        const int j = (int)((g_emu.rng >> 8) % (unsigned)(i + 1));
        std::swap(g_emu.perm[i], g_emu.perm[j]);
    }
}
inline void emu_switch_to(int nx)
{
    const int me = g_emu.cur;
    g_emu.cur = nx;
    threadIdx.x = g_emu.base + (unsigned)nx;
    swapcontext(&g_emu.lane[me], &g_emu.lane[nx]);
}
inline void emu_sync()
{
    if (++g_emu.pos == 32) {
        g_emu.pos = 0;
        emu_perm();
    }
    emu_switch_to(g_emu.perm[g_emu.pos]);
}
inline unsigned emu_lane() { return (unsigned)g_emu.cur; }

inline void __syncwarp(unsigned = 0xffffffffu) { emu_sync(); }
template <class T>
inline T emu_read(T v, int src)
{
    uint64_t u = 0;
    memcpy(&u, &v, sizeof(T));
    g_emu.xch[emu_lane()] = u;
    emu_sync();
    const uint64_t r = g_emu.xch[src & 31];
    emu_sync();
    T out;
    memcpy(&out, &r, sizeof(T));
    return out;
}
template <class T>
inline T __shfl_sync(unsigned, T v, int src) { return emu_read(v, src); }
template <class T>
inline T __shfl_up_sync(unsigned, T v, unsigned d)
{
    const int l = (int)emu_lane();
    return emu_read(v, l >= (int)d ? l - (int)d : l);
}
inline unsigned __ballot_sync(unsigned, int pred)
{
    g_emu.xch[emu_lane()] = pred ? 1u : 0u;
    emu_sync();
    unsigned m = 0;
    for (int i = 0; i < 32; ++i) m |= (unsigned)g_emu.xch[i] << i;
    emu_sync();
    return m;
}
inline int __any_sync(unsigned m, int p) { return __ballot_sync(m, p) != 0; }
inline int __ffs(unsigned x) { return x ? __builtin_ctz(x) + 1 : 0; }
inline int __clz(unsigned x) { return x ? __builtin_clz(x) : 32; }
inline uint32_t __funnelshift_r(uint32_t lo, uint32_t hi, uint32_t sh)
{
    sh &= 31;
    return sh ? (lo >> sh) | (hi << (32 - sh)) : lo;
}
template <class T>
inline T __ldg(const T *p) { return *p; }

inline void emu_lane_entry()
{
    (*g_emu.fn)();
    g_emu.done[g_emu.cur] = true;
    if (++g_emu.ndone == 32) setcontext(&g_emu.main);
    int nx = -1;
    for (int k = 1; k <= 32 && nx < 0; ++k) {
        const int p = (g_emu.pos + k) & 31;
        if (!g_emu.done[g_emu.perm[p]]) {
            nx = g_emu.perm[p];
            g_emu.pos = p;
        }
    }
    g_emu.cur = nx;
    threadIdx.x = g_emu.base + (unsigned)nx;
    setcontext(&g_emu.lane[nx]);
}

// Runs fn as one warp whose threads are base .. base+31.
inline void emu_run_warp(unsigned base, unsigned seed, std::function<void()> fn)
{
    static char *stacks = static_cast<char *>(malloc(32 * 256 * 1024));
    g_emu.fn = &fn;
    g_emu.ndone = 0;
    g_emu.base = base;
    g_emu.pos = 0;
    g_emu.rng = seed * 2654435761u + 1u;
    emu_perm();
    for (int l = 0; l < 32; ++l) {
        g_emu.done[l] = false;
        getcontext(&g_emu.lane[l]);
        g_emu.lane[l].uc_stack.ss_sp = stacks + (size_t)l * 256 * 1024;
        g_emu.lane[l].uc_stack.ss_size = 256 * 1024;
        g_emu.lane[l].uc_link = nullptr;
        makecontext(&g_emu.lane[l], emu_lane_entry, 0);
    }
    g_emu.cur = g_emu.perm[0];
    threadIdx.x = base + (unsigned)g_emu.cur;
    swapcontext(&g_emu.main, &g_emu.lane[g_emu.cur]);
}
