// gpx_explore.cu -- GB300 (sm_103a) on-the-fly state-space exploration.
//
// One persistent cooperative kernel explores a network of LTSs level by level
// (breadth-first), replacing the reference's host relaunch loop
// (GPUexplore.cu:2109-2142) and its gather / gather_por kernels
// (GPUexplore.cu:756-1189, 1191-1733):
//
//  * Frontier: all visited states live in an append-only state store in HBM
//    (the BFS queue); level L is the index range [lo, hi).  Warps claim chunks
//    of the range with one atomic, stage a batch of states in shared memory and
//    expand them.  The reference instead sweeps the whole hash table for
//    NEW-flagged entries (GPUexplore.cu:812-855).
//  * Successor generation: a batch's (state, process) pairs are spread over the
//    warp's lanes.  A lane decodes its process's local state, emits the local
//    successors, and resolves the synchronisation rules it leads (it is the
//    lowest participant) by looking up the other participants' transition
//    groups, then enumerates the rule's Cartesian product (GPUexplore.cu:904-1122).
//    Successors go through a per-warp queue in shared memory and are probed 32
//    at a time, one per lane, fully converged.
//  * Visited set: a bucketised multi-choice hash table of 32/64/128-bit slots;
//    a bucket is one 32-byte DRAM sector (64 bytes for 128-bit slots), read with
//    one 256-bit load; insertion claims the first empty slot in probe order with
//    one atomicCAS of the whole key, so a state is stored exactly once without
//    locks (the reference writes a multi-word vector word by word,
//    GPUexplore.cu:393-440).
//  * Levels end at a grid barrier whose last arriver closes the level (records
//    its count, checks violations, the state budget and errors).  Every wait is
//    bounded and reports GPX_ERR_TIMEOUT instead of hanging.
//  * Cluster POR (GPUexplore.cu:1345-1675): per state, per-process clusters,
//    proviso bits, closure and the smallest valid cluster are computed by the
//    warp; with the cycle proviso a first grid-wide pass looks every successor
//    up in the table (which holds exactly the states of earlier levels) before a
//    second pass inserts the kept successors.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cinttypes>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "gpx.h"
#include "gpx_model.h"

#include "gpx_device.cuh"
#include "gpx_live.h"

namespace gpx {

// States per work claim of a level of `cnt` states.  Claims shrink with the
// level so that small levels spread over every warp instead of queueing behind
// a few long batches, but never below a full batch: a level that fits in one
// batch per warp is split into one static claim per warp, a larger one into
// claims of at least a batch.  (One-state claims from the cursor took a
// 36K-state level of the config-2 network 88 us, a 24K-state level of a
// config-3 network 70 us per phase.)
__device__ __forceinline__ unsigned int claim_of(const Params &P, unsigned long long cnt) {
    unsigned long long per = cnt / ((unsigned long long)P.total_warps * 4ull);
    if (cnt <= (unsigned long long)P.total_warps * P.batch_states)
        per = (cnt + P.total_warps - 1) / P.total_warps;
    else if (per < P.batch_states)
        per = P.batch_states;
    return (unsigned int)(per < 1 ? 1 : (per > 4096 ? 4096 : per));
}

// What a close decided: the next phase, the end of its level, and whether the
// kernel stops (done, paused or failed).
struct Closed {
    unsigned long long hi;
    unsigned int phase, stop;
};

// Close the phase that every block has just finished (run by the last block to
// arrive at the barrier, with all other blocks waiting).
template <class K, int MODE> __device__ Closed close_phase(const Params &P) {
    Ctrl *c = P.ctrl;
    // every field the close reads, loaded together before any store: one round
    // trip to L2 instead of one per branch (config 1: 2.40 -> 2.33 ms)
    const unsigned int ph = vload(&c->phase);
    const unsigned long long ovf = vload(&c->overflow_count), hi = vload(&c->hi), sc = vload(&c->store_count);
    const unsigned int nlev = vload(&c->nlevels), lvl = vload(&c->level), ll = vload(&c->launch_levels),
                       err_read = vload(&c->error), viol = vload(&c->violation);
    if (MODE == MODE_PROVISO && ph == PH_DECIDE) {
        c->phase = PH_EXPAND;
        c->cursor = 0;
        return {hi, PH_EXPAND, err_read != 0};
    }
    if (ph == PH_PLACE) { // the overflowed keys of this level are placed
        c->place_ns += globaltimer() - c->place_t0;
        c->overflow_count = 0;
    } else if (ovf) {
        if (ovf <= P.overflow_cap && !err_read) {
            // The level's inserts are done.  The exploration kernel returns and
            // place_kernel places the overflowed keys with every warp (PH_PLACE),
            // then closes the level; the relaunch continues with the next one.
            // (A phase of the persistent kernel would cost its hot loop
            // registers: the placement code stays out of it.)
            c->phase = PH_PLACE;
            c->cursor = 0;
            c->place_t0 = globaltimer();
            c->overflowed += ovf;
            c->place_blocks = 0;
            if (P.claim) P.claim[0]++; // a new claim epoch (the counter survives runs)
            c->pause = 1;
            return {hi, PH_PLACE, 1u};
        }
        set_error(c, GPX_ERR_TABLE_FULL); // more keys than the overflow list holds
        c->overflow_count = 0;
    }
    // placement or a full overflow list may have recorded an error since
    const unsigned int err0 = (ph == PH_PLACE || ovf) ? vload(&c->error) : err_read;
    unsigned long long newhi = sc;
    if (newhi > P.store_cap) newhi = P.store_cap;
    unsigned long long cnt = newhi - hi;
    unsigned int err = err0;
    if (cnt) {
        if (nlev < kMaxLevels) {
            P.levels[nlev] = cnt;
            c->nlevels = nlev + 1;
        } else {
            set_error(c, GPX_ERR_UNSUPPORTED);
            err = GPX_ERR_UNSUPPORTED;
        }
    }
    c->level = lvl + 1;
    c->launch_levels = ll + 1;
    constexpr unsigned int kGoOn = 0xFFFFFFFFu;
    unsigned int stop = kGoOn;
    if (err)
        stop = GPX_STOP_ERROR;
    else if (viol)
        stop = GPX_STOP_VIOLATION;
    else if (cnt == 0)
        stop = GPX_STOP_DONE;
    else if (P.max_states && newhi >= P.max_states)
        stop = GPX_STOP_BUDGET;
    if (stop != kGoOn) {
        c->done = 1;
        c->stop = stop;
    }
    const unsigned int next = (MODE == MODE_PROVISO) ? PH_DECIDE : PH_EXPAND;
    c->lo = hi;
    c->hi = newhi;
    c->cursor = 0;
    c->phase = next;
    c->claim = claim_of(P, cnt);
    bool pause = false;
    if (P.levels_per_launch && ll + 1 >= P.levels_per_launch && stop == kGoOn) {
        c->pause = 1;
        pause = true;
    }
    return {newhi, next, (stop != kGoOn || pause) ? 1u : 0u};
}

// What a block needs of the current phase, read from the control block once
// per block (by the barrier thread) instead of by every warp.
struct LevelView {
    unsigned long long lo, hi;
    unsigned int claim, phase, stop;
};

__device__ __forceinline__ void read_view(const Ctrl *c, LevelView &v) {
    v.lo = vload(&c->lo);
    v.hi = vload(&c->hi);
    v.claim = vload(&c->claim);
    v.phase = vload(&c->phase);
    v.stop = vload(&c->done) | vload(&c->pause) | vload(&c->error);
}

// The barrier word the closer publishes: generation << 48 | stop << 47 |
// phase << 45 | the level's end.  Waiters take the next phase from it instead
// of reading the control block after the release (one L2 round trip less per
// phase): the level's start is the previous end (or unchanged, from a decide
// pass to its expand pass) and the claim size follows from the level's size
// exactly as the closer computes it.  A phase field of 3 (an end past 2^45)
// sends them to the control block.
constexpr unsigned long long kEndMask = (1ull << 45) - 1ull;

__device__ __forceinline__ unsigned long long phase_word(unsigned long long gen, const Closed &r) {
    const unsigned int phase = r.hi > kEndMask ? 3u : r.phase;
    return (gen << 48) | ((unsigned long long)(r.stop != 0) << 47) | ((unsigned long long)phase << 45) |
           (r.hi & kEndMask);
}

template <int MODE> __device__ __forceinline__ void next_view(const Params &P, unsigned long long w, LevelView &v) {
    const unsigned int phase = (unsigned int)(w >> 45) & 3u;
    if (phase == 3u) {
        read_view(P.ctrl, v);
        return;
    }
    if (!(MODE == MODE_PROVISO && v.phase == PH_DECIDE && phase == PH_EXPAND)) { // a new level
        v.lo = v.hi;
        v.hi = w & kEndMask;
        v.claim = claim_of(P, v.hi - v.lo);
    }
    v.phase = phase;
    v.stop = (unsigned int)(w >> 47) & 1u;
}

// Grid-wide barrier; the last block to arrive closes the phase.  The wait is
// bounded: after timeout_ns it records GPX_ERR_TIMEOUT and returns.  Thread 0
// then refreshes the block's view of the next phase.
template <class K, int MODE> __device__ void grid_barrier(const Params &P, LevelView &view) {
    __syncthreads();
    if (threadIdx.x == 0) {
        Ctrl *c = P.ctrl;
        const unsigned long long w0 = vload(&c->bar_word);
        // The arrival releases this block's writes of the phase (its warps'
        // writes are ordered before it by the block barrier) and acquires the
        // earlier arrivals'; the closer's release store of the barrier word
        // publishes the close to the waiters' acquire loads.  (Full fences
        // around plain atomics did the same, 2.5% slower per level on config 1.)
        unsigned int arrived;
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(arrived) : "l"(&c->bar_count) : "memory");
        unsigned long long w;
        if (arrived == gridDim.x - 1) {
            w = phase_word((w0 >> 48) + 1ull, close_phase<K, MODE>(P));
            c->bar_count = 0;
            asm volatile("st.release.gpu.global.u64 [%0], %1;" :: "l"(&c->bar_word), "l"(w) : "memory");
        } else { // bounded wait for the close
            uint64_t t0 = globaltimer();
            // polls at most 128 ns apart (512: config 1 2.35 -> 2.39 ms per ten rings)
            unsigned int ns = 32;
            for (;;) {
                asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(w) : "l"(&c->bar_word) : "memory");
                if ((w >> 48) != (w0 >> 48)) break;
                __nanosleep(ns);
                if (ns < 128) ns <<= 1;
                if (globaltimer() - t0 > P.timeout_ns) {
                    set_error(c, GPX_ERR_TIMEOUT);
                    atomicMax(&c->timeout_at, 1u);
                    w = 3ull << 45; // the control block: its error stops the kernel
                    break;
                }
            }
        }
        next_view<MODE>(P, w, view);
    }
    __syncthreads();
}

// The placement phase (PH_PLACE), run after a level whose inserts left keys in
// the overflow list: warp gw places entries gw, gw + warps, ... (the table is
// quiescent: the exploration kernel has returned).  A claim table lets only the
// first entry of each distinct key place it.  The last block to finish closes
// the level.  Launched after every exploration launch; it returns at once
// unless the level is waiting for placement.
template <class K, int MODE> __global__ void __launch_bounds__(256) place_kernel(Params P) {
    Ctrl *c = P.ctrl;
    if (vload(&c->phase) != PH_PLACE || vload(&c->error)) return;
    const uint32_t lane = threadIdx.x & 31;
    const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    const unsigned long long gw = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const unsigned long long n = vload(&c->overflow_count);
    const unsigned long long epoch = P.claim ? vload(P.claim) : 0;
    K *table = (K *)P.table;
    unsigned long long moves = 0, inserts = 0;
    for (unsigned long long k = gw; k < n && k < P.overflow_cap; k += warps) {
        const K x = KT<K>::load((const K *)P.overflow + k);
        int mine = 1;
        if (P.claim && lane == 0)
            mine = claim_overflow<K>(P.claim, P.claim_cap, epoch, (const K *)P.overflow, k, x,
                                     KT<K>::hash(x, P.seed ^ 0xC1A1Full));
        if (!__shfl_sync(kFull, mine, 0)) continue; // a later entry of a key already claimed
        const int r = place_warp<K>(table, P.nbuckets, x, P.seed, lane, moves);
        if (r == 2) {
            if (lane == 0) set_error(c, GPX_ERR_TABLE_FULL);
        } else if (r == 1 && lane == 0) { // a new state: the store records it for the next level
            const unsigned long long idx = atomicAdd(&c->store_count, 1ull);
            if (idx < P.store_cap) {
                ((K *)P.store)[idx] = x;
                if (P.label) P.label[idx] = 0; // its inserting move is not kept: nothing is pruned from it
            } else {
                set_error(c, GPX_ERR_STORE_FULL);
            }
            inserts++;
        }
    }
    if (lane == 0 && moves) atomicAdd(&c->evictions, moves);
    if (lane == 0 && inserts) atomicAdd(&c->inserts, inserts);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&c->place_blocks, 1u) == gridDim.x - 1) { // the last block: every key is placed
            __threadfence();
            (void)close_phase<K, MODE>(P);
        }
    }
}

// Plain mode: 4 blocks per SM (64 registers).  The POR modes: 3 blocks per SM,
// whose 85 registers leave them without spills (config 3: 79.7 vs 80.5 ms with
// 4 blocks and 124-172 bytes of spills).
template <class K, int MODE>
__global__ void __launch_bounds__(256, MODE == MODE_PLAIN ? 4 : 3) explore_kernel(Params P) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ LevelView view;
    const uint32_t *model = P.model;
    size_t model_bytes = 0;
    if (P.model_in_smem) {
        uint32_t *m = (uint32_t *)smem;
        for (uint32_t i = threadIdx.x; i < P.model_words; i += blockDim.x) m[i] = __ldg(P.model + i);
        model = m;
        model_bytes = ((size_t)P.model_words * 4 + 127) & ~(size_t)127;
    }
    WarpScratch<K, MODE> *wsall = (WarpScratch<K, MODE> *)(smem + model_bytes);
    WarpScratch<K, MODE> &ws = wsall[threadIdx.x >> 5];
    Ctrl *c = P.ctrl;
    if (threadIdx.x == 0) read_view(c, view);
    __syncthreads();

    Explorer<K, MODE> E(P, model, ws);
    const uint32_t n = E.M.n;
    uint32_t Bmax = WarpScratch<K, MODE>::kPairs / n;
    if (Bmax > 32) Bmax = 32;
    if (Bmax < 1) Bmax = 1;
    // every warp's first claim of a phase is static (warp gw takes
    // [gw * claim, (gw + 1) * claim)); the cursor hands out the rest
    const unsigned long long gw = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    while (!view.stop) {
        const unsigned long long lo = view.lo, nlev = view.hi - view.lo;
        const unsigned int claim = view.claim;
        const uint32_t B = claim < Bmax ? claim : Bmax;
        const bool decide = (MODE == MODE_PROVISO) && view.phase == PH_DECIDE;
        const unsigned long long static_end = (unsigned long long)P.total_warps * claim;
        unsigned long long base = gw * claim, size = claim;
        while (base < nlev) {
            unsigned long long end = base + size < nlev ? base + size : nlev;
            for (unsigned long long b = base; b < end; b += B) {
                uint32_t cnt = (uint32_t)((end - b) < B ? (end - b) : B);
                unsigned long long left = end - b - cnt;
                E.batch(lo + b, cnt, b, decide, (uint32_t)(left < B ? left : B));
            }
            if (static_end >= nlev) break;
            base = nlev;
            // guided self-scheduling: a quarter of a fair share of what is left
            // (between one full batch and `claim`), so the level drains in ever
            // smaller claims instead of ending on a few warps busy with full-size
            // ones; read before contending
            if (E.lane == 0) {
                const unsigned long long cur = vload(&c->cursor);
                if (static_end + cur < nlev && !vload(&c->error)) {
                    unsigned long long g = (nlev - static_end - cur) / (4ull * P.total_warps);
                    size = g < B ? B : (g > claim ? claim : g);
                    base = static_end + atomicAdd(&c->cursor, size);
                }
            }
            base = __shfl_sync(kFull, base, 0);
            size = __shfl_sync(kFull, size, 0);
        }
        E.flush_level();
        grid_barrier<K, MODE>(P, view);
    }
    E.flush_counters();
}

// Reset the control block to level 0 = {initial state} and insert the
// all-zero initial state (GPUexplore.cu:668-682).
// Tagged slots: the run's generation is the device counter *P.gen stepped by
// one, or 1 when the table was just zeroed (`cleared`).
template <class K> __global__ void init_kernel(Params P, unsigned int first_phase, unsigned int cleared) {
    Ctrl *c = P.ctrl;
    for (unsigned int i = threadIdx.x; i < sizeof(Ctrl) / 4; i += blockDim.x) ((unsigned int *)c)[i] = 0;
    __syncthreads();
    if (threadIdx.x != 0) return;
    c->store_count = 1;
    c->hi = 1;
    c->nlevels = 1;
    c->claim = 1;
    c->phase = first_phase;
    if (P.gen) {
        c->tag = cleared ? 1u : (unsigned int)*P.gen + 1u;
        *P.gen = c->tag;
    }
    K key = KT<K>::initial(c->tag);
    unsigned int probes = 0;
    find_or_insert<K>((K *)P.table, P.nbuckets, key, KT<K>::hash(key, P.seed), probes);
    ((K *)P.store)[0] = key;
    if (P.label) P.label[0] = 0;
    P.levels[0] = 1;
}

// After the last exploration launch of a graph-driven run: decide on the
// device whether another launch follows (the host relaunch loop's test,
// without the round trip), and rearm the -k budget if so.
__global__ void relaunch_kernel(Ctrl *c, cudaGraphConditionalHandle loop) {
    unsigned int more = !(c->done || c->error);
    c->launches++;
    if (more && c->launches >= kMaxLaunches) { // unreachable: each launch closes >= 1 of <= kMaxLevels levels
        set_error(c, GPX_ERR_UNSUPPORTED);
        c->done = 1;
        c->stop = GPX_STOP_ERROR;
        more = 0;
    }
    if (more) {
        c->pause = 0;
        c->launch_levels = 0;
    }
    __threadfence();
    cudaGraphSetConditional(loop, more);
}

// Order-independent hash of the visited set over the state-vector words
// (the sum of per-state key hashes; the oracle computes the same sum).  The
// state count is `count`, or min(*count_dev, cap) when count_dev is given (a
// graph captured before the count is known).
template <class K>
__global__ void set_hash_kernel(const K *store, unsigned long long count, const unsigned long long *count_dev,
                                unsigned long long cap, uint32_t words, unsigned long long *out) {
    if (count_dev) count = *count_dev < cap ? *count_dev : cap;
    auto term = [words](const K &key) {
        uint32_t w[4];
        KT<K>::words(key, w);
        uint64_t h = 0x9E3779B97F4A7C15ull;
        for (uint32_t j = 0; j < words; j += 2) {
            uint64_t cc = w[j];
            if (j + 1 < words) cc |= (uint64_t)w[j + 1] << 32;
            h = mix64(h ^ cc);
        }
        return h;
    };
    unsigned long long acc = 0;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    for (; i + 3 * stride < count; i += 4 * stride) { // four loads in flight before any hashing
        K k[4];
#pragma unroll
        for (int u = 0; u < 4; u++) k[u] = KT<K>::load(store + i + u * stride);
#pragma unroll
        for (int u = 0; u < 4; u++) acc += term(k[u]);
    }
    for (; i < count; i += stride) acc += term(KT<K>::load(store + i));
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

// Occupied slots of the table (count_states, GPUexplore.cu:687-704); slots of
// another generation are free.
template <class K>
__global__ void count_kernel(const K *table, unsigned long long slots, const Ctrl *c, unsigned long long *out) {
    const uint32_t tag = c->tag;
    unsigned long long acc = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < slots;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        K k = KT<K>::load(table + i);
        acc += KT<K>::empty(k, tag) ? 0 : 1;
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

// Convert store keys to state-vector words on the device (for collection).
template <class K>
__global__ void words_kernel(const K *store, unsigned long long count, uint32_t words, uint32_t *out) {
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < count;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t w[4];
        KT<K>::words(KT<K>::load(store + i), w);
        for (uint32_t j = 0; j < words; j++) out[i * words + j] = w[j];
    }
}

} // namespace gpx

// ========================================================================= host

using namespace gpx;

namespace {

const char *kStatusStrings[] = {"ok",
                                "input network does not exist or is malformed",
                                "no CUDA compatible GPU detected",
                                "CUDA runtime error",
                                "problem with hash table",
                                "device-side wait timed out",
                                "invalid argument",
                                "model outside the supported limits",
                                "state store full",
                                "out of memory"};

struct KernelSet {
    void (*explore[3])(Params);
    void (*place[3])(Params);
    void (*init)(Params, unsigned int, unsigned int);
    void (*set_hash)(cudaStream_t, int blocks, const void *store, unsigned long long count,
                     const unsigned long long *count_dev, unsigned long long cap, uint32_t words,
                     unsigned long long *out);
    void (*count)(cudaStream_t, int blocks, const void *table, unsigned long long slots, const Ctrl *c,
                  unsigned long long *out);
    size_t scratch_bytes[3];
    uint32_t slot_bytes, bucket_slots;
};

template <class K>
void launch_set_hash(cudaStream_t st, int blocks, const void *store, unsigned long long count,
                     const unsigned long long *count_dev, unsigned long long cap, uint32_t words,
                     unsigned long long *out) {
    set_hash_kernel<K><<<blocks, 256, 0, st>>>((const K *)store, count, count_dev, cap, words, out);
}

template <class K>
void launch_count(cudaStream_t st, int blocks, const void *table, unsigned long long slots, const Ctrl *c,
                  unsigned long long *out) {
    count_kernel<K><<<blocks, 256, 0, st>>>((const K *)table, slots, c, out);
}

template <class K> KernelSet kernels_for() {
    KernelSet s;
    s.set_hash = launch_set_hash<K>;
    s.count = launch_count<K>;
    s.explore[0] = explore_kernel<K, MODE_PLAIN>;
    s.explore[1] = explore_kernel<K, MODE_POR>;
    s.explore[2] = explore_kernel<K, MODE_PROVISO>;
    s.place[0] = place_kernel<K, MODE_PLAIN>;
    s.place[1] = place_kernel<K, MODE_POR>;
    s.place[2] = place_kernel<K, MODE_PROVISO>;
    s.init = init_kernel<K>;
    s.scratch_bytes[0] = sizeof(WarpScratch<K, MODE_PLAIN>);
    s.scratch_bytes[1] = sizeof(WarpScratch<K, MODE_POR>);
    s.scratch_bytes[2] = sizeof(WarpScratch<K, MODE_PROVISO>);
    s.slot_bytes = sizeof(K);
    s.bucket_slots = KT<K>::kSlots;
    return s;
}

#define GPX_CUDA(call)                                                                                        \
    do {                                                                                                      \
        cudaError_t _e = (call);                                                                              \
        if (_e != cudaSuccess) {                                                                              \
            fprintf(stderr, "gpx: %s failed: %s\n", #call, cudaGetErrorString(_e));                         \
            return (_e == cudaErrorMemoryAllocation) ? GPX_ERR_NOMEM : GPX_ERR_CUDA;                          \
        }                                                                                                     \
    } while (0)

} // namespace

// Everything a captured run depends on: the graph is replayed while it is unchanged.
struct GraphKey {
    Params P;
    void (*kern)(Params);
    void (*place)(Params);
    int place_blocks;
    int blocks, threads;
    size_t smem;
    unsigned int first_phase;
    uint32_t key_words;
    int collect;
    void *log_count;
    int clear; // the run zeroes the table first
    int set_hash; // the run ends with the set-hash pass
};
constexpr uint32_t kGraphLevels = 4096; // level counts read back by the graph itself

struct gpx_explorer {
    gpx_options o;
    gpx_model model;
    int kind = 0; // 0: 32-bit, 1: 64-bit, 2: 128-bit, 3: 128-bit slots with a run generation
    KernelSet ks;
    int mode = MODE_PLAIN;
    int property = GPX_PROP_NONE;
    cudaDeviceProp prop;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    void *d_table = nullptr;
    unsigned long long nbuckets = 0, slots = 0;
    size_t table_bytes = 0;
    void *d_store = nullptr;
    unsigned long long store_cap = 0;
    uint32_t *d_model = nullptr;
    size_t model_cap_words = 0;
    uint32_t *d_sel = nullptr;
    uint32_t *d_label = nullptr; // plain mode with prune_commuting: inserting move per store position
    void *d_overflow = nullptr; // keys whose probe sequence was full during a level
    unsigned long long overflow_cap = 0;
    unsigned long long *d_claim = nullptr; // claim table of the placement phase (epoch counter + entries)
    unsigned long long claim_cap = 0;
    unsigned long long *d_levels = nullptr;
    unsigned long long *d_scalar = nullptr;
    Ctrl *d_ctrl = nullptr;
    Ctrl *h_ctrl = nullptr;
    int blocks = 0, threads = 0;
    size_t smem = 0;
    bool model_in_smem = false;
    unsigned long long last_count = 0, last_lo = 0, last_hi = 0;
    uint32_t bits_statevector = 0;
    gpx_por_model *d_por_model = nullptr; // learned proposal (por == 2)
    bool have_por_model = false;
    gpx_por_log_row *d_log = nullptr;     // candidate log (decide pass)
    unsigned long long *d_log_count = nullptr;
    unsigned long long log_cap = 0;
    uint32_t log_every = 0;
    // a run as one CUDA graph (launch_graph), rebuilt when its key changes
    GraphKey graph_key[2];                   // [clear]: runs that zero the table, and the others
    cudaGraph_t graph[2] = {nullptr, nullptr};
    cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};
    cudaStream_t st_body = nullptr;          // captures the body of the launch loop
    unsigned long long *h_levels = nullptr;  // pinned: the first kGraphLevels level counts
    unsigned long long *h_scalar = nullptr;  // pinned: set hash, table count
    LiveScratch live;                        // accepting-cycle check (liveness)
    size_t saved_fetch = 0;                  // the context's L2 fetch granularity limit before the first run
    bool fetch_saved = false;
    // tagged slots (kind 3): generation of the table's newest keys (0: contents
    // unknown, clear before the next run); the device steps its own copy
    unsigned int gen = 0;
};

namespace {

// gpx_options.por: 1 cample, 2 cample with the learned proposal, 3 ample, 4 stubborn
uint32_t por_kind_of(int por) { return por == 3 ? POR_AMPLE : (por == 4 ? POR_STUBBORN : POR_CAMPLE); }

// Checks every entry point that takes gpx_options makes before it touches the
// device, so that the same options are accepted or refused everywhere.  Sizes
// are bounded so that no byte count derived from them overflows 64 bits.
int check_options(const gpx_options *o) {
    if (!o || o->struct_size != sizeof(gpx_options)) return GPX_ERR_INVALID;
    if (o->bucket_bytes != 0 && o->bucket_bytes != 32) return GPX_ERR_INVALID;
    if (o->por < 0 || o->por > 4) return GPX_ERR_INVALID;
    if (o->property < GPX_PROP_NONE || o->property > GPX_PROP_LIVENESS) return GPX_ERR_INVALID;
    if (o->threads < 0 || o->threads % 32 || o->threads > 256) return GPX_ERR_INVALID;
    if (o->q_words > (1ull << 60) || o->store_states > (1ull << 58)) return GPX_ERR_INVALID;
    return GPX_OK;
}

// Slot form for a state width.  A table the explorer keeps across runs takes
// the generation-tagged form when the state fits its 112 bits.
int select_kind(uint32_t state_bits, bool reusable) {
    if (state_bits <= 31) return 0;
    if (state_bits <= 63) return 1;
    return (reusable && state_bits <= 112) ? 3 : 2;
}

KernelSet kernels_of(int kind) {
    switch (kind) {
    case 0: return kernels_for<K32>();
    case 1: return kernels_for<K64>();
    case 2: return kernels_for<K128>();
    default: return kernels_for<K128G>();
    }
}

int load_text(const std::string &path, gpx_model **out) {
    std::ifstream f(path);
    if (!f) return GPX_ERR_PARSE;
    std::stringstream ss;
    ss << f.rdbuf();
    gpx_model *m = new gpx_model;
    std::string err = parse_gpf_text(ss.str(), &m->gpf);
    if (err.empty()) err = decode_gpf(m->gpf, &m->dec);
    if (!err.empty()) {
        fprintf(stderr, "gpx: %s: %s\n", path.c_str(), err.c_str());
        int code = err.rfind("UNSUPPORTED", 0) == 0 ? GPX_ERR_UNSUPPORTED : GPX_ERR_PARSE;
        delete m;
        return code;
    }
    *out = m;
    return GPX_OK;
}

int configure_launch(gpx_explorer *ex) {
    const size_t model_bytes = ex->model.dec.words.size() * 4;
    int threads = ex->o.threads > 0 ? ex->o.threads : 256;
    if (threads % 32 || threads > 256) return GPX_ERR_INVALID;
    const size_t smem_limit = ex->prop.sharedMemPerBlockOptin;
    size_t scratch = (size_t)(threads / 32) * ex->ks.scratch_bytes[ex->mode];
    size_t mb = (model_bytes + 127) & ~(size_t)127;
    ex->model_in_smem = (mb + scratch <= smem_limit) && model_bytes <= 96 * 1024;
    ex->smem = scratch + (ex->model_in_smem ? mb : 0);
    if (ex->smem > smem_limit) return GPX_ERR_UNSUPPORTED;
    for (int md = 0; md < 3; md++)
        GPX_CUDA(cudaFuncSetAttribute((const void *)ex->ks.explore[md], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)ex->smem));
    int per_sm = 0;
    GPX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)ex->ks.explore[ex->mode],
                                                           threads, ex->smem));
    if (per_sm < 1) return GPX_ERR_UNSUPPORTED;
    int max_blocks = per_sm * ex->prop.multiProcessorCount;
    int blocks = ex->o.blocks > 0 ? std::min(ex->o.blocks, max_blocks) : max_blocks;
    ex->blocks = std::max(1, blocks);
    ex->threads = threads;
    return GPX_OK;
}

int upload_model(gpx_explorer *ex) {
    const std::vector<uint32_t> &w = ex->model.dec.words;
    if (w.size() > ex->model_cap_words) {
        if (ex->d_model) cudaFree(ex->d_model);
        ex->d_model = nullptr;
        GPX_CUDA(cudaMalloc(&ex->d_model, w.size() * 4));
        ex->model_cap_words = w.size();
    }
    GPX_CUDA(cudaMemcpyAsync(ex->d_model, w.data(), w.size() * 4, cudaMemcpyHostToDevice, ex->st));
    return GPX_OK;
}

// States in a warp's full batch: its (state, process) pairs over the processes.
uint32_t batch_states_of(int mode, size_t nprocs) {
    const size_t pairs = mode == MODE_PLAIN ? kPairMax : kPairMaxPor;
    const size_t b = nprocs ? pairs / nprocs : 1;
    return (uint32_t)std::max<size_t>(1, std::min<size_t>(32, b));
}

Params make_params(gpx_explorer *ex) {
    Params P;
    memset(&P, 0, sizeof P);
    P.table = ex->d_table;
    P.nbuckets = ex->nbuckets;
    P.store = ex->d_store;
    P.store_cap = ex->store_cap;
    P.model = ex->d_model;
    P.model_words = (uint32_t)ex->model.dec.words.size();
    P.model_in_smem = ex->model_in_smem;
    P.sel = ex->d_sel;
    P.label = ex->mode == MODE_PLAIN ? ex->d_label : nullptr;
    P.overflow = ex->d_overflow;
    P.overflow_cap = ex->overflow_cap;
    P.claim = ex->d_claim;
    P.claim_cap = ex->claim_cap;
    P.levels = ex->d_levels;
    P.ctrl = ex->d_ctrl;
    P.seed = ex->o.seed;
    P.max_states = ex->o.max_states;
    P.timeout_ns = 20ull * 1000 * 1000 * 1000;
    P.property = (uint32_t)ex->property;
    P.levels_per_launch = ex->o.kernel_iters > 0 ? (uint32_t)ex->o.kernel_iters : 0;
    P.total_warps = (uint32_t)(ex->blocks * (ex->threads / 32));
    P.batch_states = batch_states_of(ex->mode, ex->model.dec.nstates.size());
    P.learned = (ex->o.por == 2 && ex->have_por_model) ? 1u : 0u;
    P.por_kind = por_kind_of(ex->o.por);
    P.por_model = ex->have_por_model ? ex->d_por_model : nullptr;
    P.gen = ex->kind == 3 ? ex->d_scalar + 2 : nullptr;
    if (ex->d_log && ex->log_cap && ex->mode == MODE_PROVISO) {
        P.log = ex->d_log;
        P.log_count = ex->d_log_count;
        P.log_cap = ex->log_cap;
        P.log_every = ex->log_every;
    }
    return P;
}

// Grid of place_kernel: a few blocks per SM (most launches return at once).
int place_grid(const gpx_explorer *ex) { return 4 * ex->prop.multiProcessorCount; }

int count_blocks(const gpx_explorer *ex) {
    return (int)std::max<unsigned long long>(1, std::min<unsigned long long>((ex->slots + 255) / 256, 8192));
}

void destroy_graph(gpx_explorer *ex) {
    for (int c = 0; c < 2; c++) {
        if (ex->graph_exec[c]) cudaGraphExecDestroy(ex->graph_exec[c]);
        if (ex->graph[c]) cudaGraphDestroy(ex->graph[c]);
        ex->graph_exec[c] = nullptr;
        ex->graph[c] = nullptr;
    }
}

GraphKey graph_key(const gpx_explorer *ex, const Params &P, unsigned int first_phase, bool clear) {
    GraphKey k;
    memset(&k, 0, sizeof k);
    k.P = P;
    k.kern = ex->ks.explore[ex->mode];
    k.place = ex->ks.place[ex->mode];
    k.place_blocks = place_grid(ex);
    k.blocks = ex->blocks;
    k.threads = ex->threads;
    k.smem = ex->smem;
    k.first_phase = first_phase;
    k.key_words = ex->model.dec.key_words;
    k.collect = (ex->o.collect_states || ex->o.verbosity >= 2) ? 1 : 0;
    k.log_count = ex->d_log_count;
    k.clear = clear ? 1 : 0;
    k.set_hash = ex->o.set_hash ? 1 : 0;
    return k;
}

// Record one run into a graph on ex->st:
//   [zero the table] + init -> while (more) { exploration launch; placement; relaunch_kernel }
//   -> [set hash] -> read-back
// The loop's condition is set on the device by relaunch_kernel, so a -k run
// needs no host round trip between launches.
cudaError_t capture_run(gpx_explorer *ex, const GraphKey &k, cudaGraph_t *out) {
    cudaStream_t st = ex->st, sb = ex->st_body;
    bool body_open = false;
    auto record = [&]() -> cudaError_t {
        cudaError_t e;
#define GPX_CAP(call)                                                                                         \
    do {                                                                                                      \
        if ((e = (call)) != cudaSuccess) return e;                                                            \
    } while (0)
        Params P = k.P;
        GPX_CAP(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        GPX_CAP(cudaEventRecordWithFlags(ex->ev[0], st, cudaEventRecordExternal));
        if (k.clear) GPX_CAP(cudaMemsetAsync(ex->d_table, 0, ex->table_bytes, st));
        if (k.log_count) GPX_CAP(cudaMemsetAsync(k.log_count, 0, 8, st));
        ex->ks.init<<<1, 32, 0, st>>>(P, k.first_phase, (unsigned int)k.clear);
        GPX_CAP(cudaGetLastError());
        GPX_CAP(cudaEventRecordWithFlags(ex->ev[1], st, cudaEventRecordExternal));

        cudaStreamCaptureStatus cs;
        cudaGraph_t g = nullptr;
        const cudaGraphNode_t *deps = nullptr;
        const cudaGraphEdgeData *edges = nullptr;
        size_t ndeps = 0;
        GPX_CAP(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &edges, &ndeps));
        cudaGraphConditionalHandle loop;
        GPX_CAP(cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams np = {cudaGraphNodeTypeConditional}; // the rest zero-initialised
        np.conditional.handle = loop;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        GPX_CAP(cudaGraphAddNode(&node, g, deps, edges, ndeps, &np));
        GPX_CAP(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
        GPX_CAP(cudaStreamBeginCaptureToGraph(sb, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal));
        body_open = true;
        void *args[] = {&P};
        GPX_CAP(cudaLaunchCooperativeKernel((const void *)k.kern, dim3(k.blocks), dim3(k.threads), args, k.smem, sb));
        k.place<<<k.place_blocks, 256, 0, sb>>>(P); // returns at once unless a level waits for placement
        relaunch_kernel<<<1, 1, 0, sb>>>(ex->d_ctrl, loop);
        GPX_CAP(cudaGetLastError());
        cudaGraph_t body = nullptr; // owned by the conditional node
        body_open = false;
        GPX_CAP(cudaStreamEndCapture(sb, &body));

        GPX_CAP(cudaEventRecordWithFlags(ex->ev[3], st, cudaEventRecordExternal));
        GPX_CAP(cudaMemsetAsync(ex->d_scalar, 0, 16, st));
        if (k.set_hash) {
            int hb = (int)std::max<unsigned long long>(1, std::min<unsigned long long>((ex->store_cap + 255) / 256,
                                                                                      4096));
            ex->ks.set_hash(st, hb, ex->d_store, 0, &ex->d_ctrl->store_count, ex->store_cap, k.key_words,
                            ex->d_scalar);
        }
        if (k.collect) ex->ks.count(st, count_blocks(ex), ex->d_table, ex->slots, ex->d_ctrl, ex->d_scalar + 1);
        GPX_CAP(cudaGetLastError());
        GPX_CAP(cudaMemcpyAsync(ex->h_ctrl, ex->d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, st));
        GPX_CAP(cudaMemcpyAsync(ex->h_scalar, ex->d_scalar, 16, cudaMemcpyDeviceToHost, st));
        GPX_CAP(cudaMemcpyAsync(ex->h_levels, ex->d_levels, (size_t)kGraphLevels * 8, cudaMemcpyDeviceToHost, st));
#undef GPX_CAP
        return cudaStreamEndCapture(st, out);
    };
    cudaError_t e = record();
    if (e != cudaSuccess) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaGraph_t t = nullptr;
        if (body_open) cudaStreamEndCapture(sb, &t);
        if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
            t = nullptr;
            cudaStreamEndCapture(st, &t);
            if (t) cudaGraphDestroy(t);
        }
        cudaGetLastError();
    }
    return e;
}

// Run the exploration as one graph launch (built on first use or when the key changed).
int run_graph(gpx_explorer *ex, const Params &P, unsigned int first_phase, bool clear) {
    GraphKey k = graph_key(ex, P, first_phase, clear);
    const int c = clear ? 1 : 0;
    if (!ex->graph_exec[c] || memcmp(&k, &ex->graph_key[c], sizeof k) != 0) {
        if (ex->graph_exec[c]) cudaGraphExecDestroy(ex->graph_exec[c]);
        if (ex->graph[c]) cudaGraphDestroy(ex->graph[c]);
        ex->graph_exec[c] = nullptr;
        ex->graph[c] = nullptr;
        if (!ex->st_body) GPX_CUDA(cudaStreamCreateWithFlags(&ex->st_body, cudaStreamNonBlocking));
        if (!ex->h_levels) GPX_CUDA(cudaMallocHost(&ex->h_levels, (size_t)kGraphLevels * 8));
        if (!ex->h_scalar) GPX_CUDA(cudaMallocHost(&ex->h_scalar, 16));
        cudaGraph_t g = nullptr;
        cudaError_t e = capture_run(ex, k, &g);
        if (e == cudaSuccess) {
            ex->graph[c] = g;
            e = cudaGraphInstantiate(&ex->graph_exec[c], g, 0);
        }
        if (e != cudaSuccess) {
            fprintf(stderr, "gpx: building the run graph failed: %s (launch_graph = 0 runs without it)\n",
                    cudaGetErrorString(e));
            destroy_graph(ex);
            cudaGetLastError();
            return GPX_ERR_CUDA;
        }
        ex->graph_key[c] = k;
    }
    GPX_CUDA(cudaGraphLaunch(ex->graph_exec[c], ex->st));
    GPX_CUDA(cudaStreamSynchronize(ex->st));
    return GPX_OK;
}

void print_states(FILE *out, gpx_explorer *ex, const std::vector<uint32_t> &words, unsigned long long count,
                  unsigned long long unexplored_from) {
    const Gpf &g = ex->model.gpf;
    const uint32_t W = ex->model.dec.key_words;
    const uint32_t sv = (ex->bits_statevector + 31) / 32;
    unsigned long long newcount = 0;
    for (unsigned long long i = 0; i < count; i++) {
        const uint32_t *v = words.data() + i * W;
        if (i >= unexplored_from) {
            fprintf(out, "new: ");
            newcount++;
        }
        for (uint32_t p = 0; p < g.nr_procs; p++) {
            uint32_t lo = g.firstbit[p], w = g.bits_state[p];
            uint64_t x = v[lo / 32];
            if ((lo % 32) + w > 32) x |= (uint64_t)v[lo / 32 + 1] << 32;
            fprintf(out, "%u%s", (uint32_t)((x >> (lo % 32)) & ((1ull << w) - 1)), p + 1 < g.nr_procs ? "," : "");
        }
        fprintf(out, " ");
        for (uint32_t j = 0; j < sv; j++) fprintf(out, "%d ", (int)(j < W ? v[j] : 0u));
        fprintf(out, "\n");
    }
    fprintf(out, "nr. of states in hash table: %llu (%llu unexplored states)\n", count, newcount);
}

int collect_words(gpx_explorer *ex, unsigned long long count, std::vector<uint32_t> *out) {
    const uint32_t W = ex->model.dec.key_words;
    out->assign(count * W, 0);
    if (!count) return GPX_OK;
    uint32_t *d_words = nullptr;
    GPX_CUDA(cudaMalloc(&d_words, count * W * 4));
    int blocks = (int)std::min<unsigned long long>((count + 255) / 256, 4096);
    if (ex->kind == 0)
        words_kernel<K32><<<blocks, 256, 0, ex->st>>>((const K32 *)ex->d_store, count, W, d_words);
    else if (ex->kind == 1)
        words_kernel<K64><<<blocks, 256, 0, ex->st>>>((const K64 *)ex->d_store, count, W, d_words);
    else if (ex->kind == 2)
        words_kernel<K128><<<blocks, 256, 0, ex->st>>>((const K128 *)ex->d_store, count, W, d_words);
    else
        words_kernel<K128G><<<blocks, 256, 0, ex->st>>>((const K128G *)ex->d_store, count, W, d_words);
    cudaError_t e = cudaMemcpyAsync(out->data(), d_words, count * W * 4, cudaMemcpyDeviceToHost, ex->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ex->st);
    cudaFree(d_words);
    if (e != cudaSuccess) return GPX_ERR_CUDA;
    return GPX_OK;
}

} // namespace

extern "C" {

const char *gpx_status_string(int status) {
    if (status < 0 || status > GPX_ERR_NOMEM) return "unknown status";
    return kStatusStrings[status];
}

int gpx_abi_version(void) { return GPX_ABI_VERSION; }

int gpx_device_info_get(int device, gpx_device_info *info) {
    if (!info) return GPX_ERR_INVALID;
    memset(info, 0, sizeof *info);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GPX_ERR_NO_GPU;
    if (device < 0 || device >= ndev) return GPX_ERR_INVALID;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return GPX_ERR_CUDA;
    info->total_global_mem = prop.totalGlobalMem;
    info->shared_mem_per_block = (int32_t)prop.sharedMemPerBlock;
    info->shared_mem_per_sm = (int32_t)prop.sharedMemPerMultiprocessor;
    info->max_threads_per_block = prop.maxThreadsPerBlock;
    info->max_grid_size = prop.maxGridSize[0];
    info->sm_count = prop.multiProcessorCount;
    snprintf(info->name, sizeof info->name, "%s", prop.name);
    return GPX_OK;
}

void gpx_options_init(gpx_options *o) {
    memset(o, 0, sizeof *o);
    o->struct_size = sizeof *o;
    o->seed = 0x243F6A8885A308D3ull;
    o->launch_graph = 1;
    o->prune_commuting = 1;
}

int gpx_model_load(const char *path_without_ext, gpx_model **out) {
    if (!path_without_ext || !out) return GPX_ERR_INVALID;
    return load_text(std::string(path_without_ext) + ".gpf", out);
}

int gpx_model_load_file(const char *path, gpx_model **out) {
    if (!path || !out) return GPX_ERR_INVALID;
    return load_text(path, out);
}

int gpx_model_from_words(const uint32_t *words, size_t nwords, gpx_model **out) {
    if (!words || !out) return GPX_ERR_INVALID;
    gpx_model *m = new gpx_model;
    std::string err = parse_gpf_words(words, nwords, &m->gpf);
    if (err.empty()) err = decode_gpf(m->gpf, &m->dec);
    if (!err.empty()) {
        int code = err.rfind("UNSUPPORTED", 0) == 0 ? GPX_ERR_UNSUPPORTED : GPX_ERR_PARSE;
        delete m;
        return code;
    }
    *out = m;
    return GPX_OK;
}

int gpx_model_info_get(const gpx_model *m, gpx_model_info *info) {
    if (!m || !info) return GPX_ERR_INVALID;
    memset(info, 0, sizeof *info);
    const Gpf &g = m->gpf;
    info->liveness = g.liveness;
    info->nr_procs = g.nr_procs;
    info->bits_act = g.bits_act;
    info->proc_nrstates = g.proc_nrstates;
    info->bits_statevector = g.bits_statevector;
    info->nbits_offset = g.nbits_offset;
    info->max_buf_ints = g.max_buf_ints;
    info->nr_trans = g.nr_trans;
    info->state_bits = m->dec.state_bits;
    info->key_words = m->dec.key_words;
    for (uint32_t p = 0; p <= g.nr_procs; p++) info->firstbit[p] = g.firstbit[p];
    for (uint32_t p = 0; p < g.nr_procs; p++) info->bits_state[p] = g.bits_state[p];
    return GPX_OK;
}

void gpx_model_free(gpx_model *m) { delete m; }

void gpx_explorer_destroy(gpx_explorer *ex) {
    if (!ex) return;
    if (ex->fetch_saved) {
        cudaSetDevice(ex->o.device);
        cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, ex->saved_fetch);
    }
    destroy_graph(ex);
    live_free(&ex->live);
    if (ex->st_body) cudaStreamDestroy(ex->st_body);
    if (ex->h_levels) cudaFreeHost(ex->h_levels);
    if (ex->h_scalar) cudaFreeHost(ex->h_scalar);
    if (ex->d_table) cudaFree(ex->d_table);
    if (ex->d_store) cudaFree(ex->d_store);
    if (ex->d_model) cudaFree(ex->d_model);
    if (ex->d_sel) cudaFree(ex->d_sel);
    if (ex->d_label) cudaFree(ex->d_label);
    if (ex->d_overflow) cudaFree(ex->d_overflow);
    if (ex->d_claim) cudaFree(ex->d_claim);
    if (ex->d_levels) cudaFree(ex->d_levels);
    if (ex->d_scalar) cudaFree(ex->d_scalar);
    if (ex->d_ctrl) cudaFree(ex->d_ctrl);
    if (ex->h_ctrl) cudaFreeHost(ex->h_ctrl);
    if (ex->d_por_model) cudaFree(ex->d_por_model);
    if (ex->d_log) cudaFree(ex->d_log);
    if (ex->d_log_count) cudaFree(ex->d_log_count);
    for (auto &e : ex->ev)
        if (e) cudaEventDestroy(e);
    if (ex->st) cudaStreamDestroy(ex->st);
    delete ex;
}

int gpx_explorer_create(const gpx_model *model, const gpx_options *opts, gpx_explorer **out) {
    if (!model || !out) return GPX_ERR_INVALID;
    if (int bad = check_options(opts)) return bad;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GPX_ERR_NO_GPU;
    if (opts->device < 0 || opts->device >= ndev) return GPX_ERR_INVALID;
    gpx_explorer *ex = new gpx_explorer;
    ex->o = *opts;
    ex->model = *model;
    ex->property = opts->property;
    if (ex->property == GPX_PROP_SAFETY && model->gpf.liveness == 1) ex->property = GPX_PROP_LIVENESS;
    ex->mode = opts->por ? (opts->cycle_proviso ? MODE_PROVISO : MODE_POR) : MODE_PLAIN;
    // the accepting-cycle check needs the full state graph
    if (ex->property == GPX_PROP_LIVENESS && ex->mode != MODE_PLAIN) {
        delete ex;
        return GPX_ERR_UNSUPPORTED;
    }
    ex->kind = select_kind(model->dec.state_bits, true);
    ex->ks = kernels_of(ex->kind);
    ex->bits_statevector = model->gpf.bits_statevector + (opts->por ? 1u : 0u);
    int rc = GPX_OK;
    auto fail = [&](int code) {
        gpx_explorer_destroy(ex);
        return code;
    };
    if (cudaSetDevice(opts->device) != cudaSuccess) return fail(GPX_ERR_CUDA);
    if (cudaGetDeviceProperties(&ex->prop, opts->device) != cudaSuccess) return fail(GPX_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&ex->st, cudaStreamNonBlocking) != cudaSuccess) return fail(GPX_ERR_CUDA);
    for (auto &e : ex->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return fail(GPX_ERR_CUDA);
    if ((rc = configure_launch(ex)) != GPX_OK) return fail(rc);

    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return fail(GPX_ERR_CUDA);
    const size_t bucket_bytes = (size_t)ex->ks.slot_bytes * ex->ks.bucket_slots;
    size_t tb = opts->q_words ? (size_t)opts->q_words * 4 : free_b / 4;
    tb = (tb / (2 * bucket_bytes)) * (2 * bucket_bytes); // buckets are probed in pairs
    if (tb < 2 * bucket_bytes) return fail(GPX_ERR_INVALID);
    ex->table_bytes = tb;
    ex->nbuckets = tb / bucket_bytes;
    ex->slots = ex->nbuckets * ex->ks.bucket_slots;
    const bool labels = ex->mode == MODE_PLAIN && opts->prune_commuting;
    const size_t per_state = ex->ks.slot_bytes + (ex->mode == MODE_PROVISO || labels ? 4 : 0);
    unsigned long long cap = opts->store_states ? opts->store_states : ex->slots;
    size_t margin = (size_t)512 << 20;
    size_t avail = free_b > tb + margin ? free_b - tb - margin : 0;
    // compare in states, not bytes: cap * per_state could wrap for an explicit store_states
    if (cap > avail / per_state) {
        if (opts->store_states) return fail(GPX_ERR_NOMEM);
        cap = avail / per_state;
    }
    if (cap < 1) return fail(GPX_ERR_NOMEM);
    ex->store_cap = cap;
    if (cudaMalloc(&ex->d_table, tb) != cudaSuccess) return fail(GPX_ERR_NOMEM);
    if (cudaMalloc(&ex->d_store, cap * ex->ks.slot_bytes) != cudaSuccess) return fail(GPX_ERR_NOMEM);
    if (ex->mode == MODE_PROVISO && cudaMalloc(&ex->d_sel, cap * 4) != cudaSuccess) return fail(GPX_ERR_NOMEM);
    if (labels && cudaMalloc(&ex->d_label, cap * 4) != cudaSuccess) return fail(GPX_ERR_NOMEM);
    ex->overflow_cap = 1u << 16;
    if (cudaMalloc(&ex->d_overflow, ex->overflow_cap * ex->ks.slot_bytes) != cudaSuccess) return fail(GPX_ERR_NOMEM);
    ex->claim_cap = 2 * ex->overflow_cap; // entries of 16 bytes after a 16-byte epoch counter
    if (cudaMalloc(&ex->d_claim, (2 + 2 * ex->claim_cap) * 8) != cudaSuccess) return fail(GPX_ERR_NOMEM);
    if (cudaMemset(ex->d_claim, 0, (2 + 2 * ex->claim_cap) * 8) != cudaSuccess) return fail(GPX_ERR_CUDA);
    if (cudaMalloc(&ex->d_levels, (size_t)kMaxLevels * 8) != cudaSuccess) return fail(GPX_ERR_NOMEM);
    if (cudaMalloc(&ex->d_scalar, 64) != cudaSuccess) return fail(GPX_ERR_NOMEM);
    if (cudaMalloc(&ex->d_ctrl, sizeof(Ctrl)) != cudaSuccess) return fail(GPX_ERR_NOMEM);
    if (cudaMallocHost(&ex->h_ctrl, sizeof(Ctrl)) != cudaSuccess) return fail(GPX_ERR_NOMEM);
    if ((rc = upload_model(ex)) != GPX_OK) return fail(rc);
    if (cudaStreamSynchronize(ex->st) != cudaSuccess) return fail(GPX_ERR_CUDA);
    *out = ex;
    return GPX_OK;
}

int gpx_explorer_set_model(gpx_explorer *ex, const gpx_model *model) {
    if (!ex || !model) return GPX_ERR_INVALID;
    // the slot size is fixed by the table; the two 128-bit forms interchange
    const int kind = select_kind(model->dec.state_bits, true);
    if (kind != ex->kind && !(kind >= 2 && ex->kind >= 2)) return GPX_ERR_INVALID;
    int property = ex->o.property;
    if (property == GPX_PROP_SAFETY && model->gpf.liveness == 1) property = GPX_PROP_LIVENESS;
    if (property == GPX_PROP_LIVENESS && ex->mode != MODE_PLAIN) return GPX_ERR_UNSUPPORTED;
    ex->property = property;
    if (kind != ex->kind) { // the table's keys are of the other form: clear it before the next run
        ex->kind = kind;
        ex->ks = kernels_of(kind);
        ex->gen = 0;
    }
    ex->model = *model;
    ex->bits_statevector = model->gpf.bits_statevector + (ex->o.por ? 1u : 0u);
    int rc = configure_launch(ex);
    if (rc != GPX_OK) return rc;
    return upload_model(ex);
}

int gpx_explorer_run(gpx_explorer *ex, gpx_result *r) {
    if (!ex || !r) return GPX_ERR_INVALID;
    memset(r, 0, sizeof *r);
    r->struct_size = sizeof *r;
    if (cudaSetDevice(ex->o.device) != cudaSuccess) return GPX_ERR_CUDA;
    Params P = make_params(ex);
    const unsigned int first_phase = ex->mode == MODE_PROVISO ? PH_DECIDE : PH_EXPAND;
    // Hash probes are random 32-byte reads: ask L2 to fetch no more than a sector
    // per miss (unset, a miss fills 128 bytes; the request rate is the same either
    // way, the DRAM traffic is not).  Setting the limit waits for the device (a few
    // hundred microseconds), so it is set only when it differs, and the caller's
    // value comes back when the explorer is destroyed.
    size_t cur_fetch = 0;
    if (cudaDeviceGetLimit(&cur_fetch, cudaLimitMaxL2FetchGranularity) == cudaSuccess && cur_fetch != 32 &&
        cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, 32) == cudaSuccess && !ex->fetch_saved) {
        ex->saved_fetch = cur_fetch;
        ex->fetch_saved = true;
    }
    unsigned long long launches = 0;
    float kernel_ms = 0, setup_ms = 0, total_ms = 0;
    // reset: empty table, empty store, initial state (GPUexplore.cu:2091-2092).
    // Tagged slots need no clear while the generation counts up: a run's keys
    // carry its generation and older ones read as free.  The table is zeroed
    // when its contents are unknown (first run, a failed run, a change of slot
    // form) and when the 8-bit generation is spent.
    const bool tagged = ex->kind == 3;
    const bool clear = !tagged || ex->gen == 0 || ex->gen >= 255;
    const unsigned int tag = tagged ? (clear ? 1u : ex->gen + 1u) : 0u;
    ex->gen = 0; // until this run has completed
    // -v prints between launches, so it keeps the host loop
    const bool graph = ex->o.launch_graph && ex->o.verbosity <= 0;
    if (graph) {
        int rc = run_graph(ex, P, first_phase, clear);
        if (rc != GPX_OK) return rc;
        launches = ex->h_ctrl->launches;
        cudaEventElapsedTime(&setup_ms, ex->ev[0], ex->ev[1]);
        cudaEventElapsedTime(&kernel_ms, ex->ev[1], ex->ev[3]);
        total_ms = kernel_ms;
    } else {
        GPX_CUDA(cudaEventRecord(ex->ev[0], ex->st));
        if (clear) GPX_CUDA(cudaMemsetAsync(ex->d_table, 0, ex->table_bytes, ex->st));
        if (ex->d_log_count) GPX_CUDA(cudaMemsetAsync(ex->d_log_count, 0, 8, ex->st));
        ex->ks.init<<<1, 32, 0, ex->st>>>(P, first_phase, clear ? 1u : 0u);
        GPX_CUDA(cudaGetLastError());
        GPX_CUDA(cudaEventRecord(ex->ev[1], ex->st));
        void (*kern)(Params) = ex->ks.explore[ex->mode];
        void *args[] = {&P};
        for (;;) {
            GPX_CUDA(cudaEventRecord(ex->ev[2], ex->st));
            GPX_CUDA(cudaLaunchCooperativeKernel((const void *)kern, dim3(ex->blocks), dim3(ex->threads), args,
                                                 ex->smem, ex->st));
            ex->ks.place[ex->mode]<<<place_grid(ex), 256, 0, ex->st>>>(P); // a level waiting for placement
            GPX_CUDA(cudaGetLastError());
            GPX_CUDA(cudaEventRecord(ex->ev[3], ex->st));
            launches++;
            GPX_CUDA(cudaMemcpyAsync(ex->h_ctrl, ex->d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, ex->st));
            GPX_CUDA(cudaStreamSynchronize(ex->st));
            float ms = 0;
            cudaEventElapsedTime(&ms, ex->ev[2], ex->ev[3]);
            kernel_ms += ms;
            Ctrl &c = *ex->h_ctrl;
            if (ex->o.verbosity == 1) printf("%llu\n", launches - 1);
            if (ex->o.verbosity >= 2) {
                unsigned long long cnt = std::min<unsigned long long>(c.store_count, ex->store_cap);
                if (ex->o.verbosity == 2) {
                    printf("nr. of states in hash table: %llu (%llu unexplored states)\n", cnt, cnt - c.lo);
                } else {
                    std::vector<uint32_t> w;
                    int rc = collect_words(ex, cnt, &w);
                    if (rc != GPX_OK) return rc;
                    print_states(stdout, ex, w, cnt, c.lo);
                }
            }
            if (c.done || c.error) break;
            // -k budget reached: resume with a fresh launch
            c.pause = 0;
            c.launch_levels = 0;
            GPX_CUDA(cudaMemcpyAsync(&ex->d_ctrl->pause, &c.pause, sizeof(unsigned int), cudaMemcpyHostToDevice,
                                     ex->st));
            GPX_CUDA(cudaMemcpyAsync(&ex->d_ctrl->launch_levels, &c.launch_levels, sizeof(unsigned int),
                                     cudaMemcpyHostToDevice, ex->st));
        }
        cudaEventElapsedTime(&setup_ms, ex->ev[0], ex->ev[1]);
        cudaEventElapsedTime(&total_ms, ex->ev[1], ex->ev[3]);
    }
    Ctrl &c = *ex->h_ctrl;
    ex->gen = tag; // the table holds this run's keys (and older, free ones)
    r->status = c.error ? (int)c.error : GPX_OK;
    r->stopped = (int)c.stop;
    if (c.error) r->stopped = GPX_STOP_ERROR;
    r->verdict = (c.stop == GPX_STOP_VIOLATION) ? ex->property : GPX_PROP_NONE;
    unsigned long long count = std::min<unsigned long long>(c.store_count, ex->store_cap);
    r->states = count;
    r->nlevels = c.nlevels;
    r->level_counts = (uint64_t *)malloc(sizeof(uint64_t) * std::max(1u, c.nlevels));
    r->lookups = c.lookups;
    r->transitions = c.inserts_lookups; // successors sent to the table for insertion
    r->probes = c.probes;
    r->inserts = c.inserts;
    r->evictions = c.evictions;
    r->pruned = c.pruned;
    r->overflowed = c.overflowed;
    r->evict_ms = c.place_ns * 1e-6;
    r->expanded = c.expanded;
    r->launches = launches;
    r->kernel_ms = kernel_ms;
    r->explore_ms = total_ms;
    r->setup_ms = setup_ms;
    r->key_words = ex->model.dec.key_words;
    r->table_slots = ex->slots;
    r->slot_bytes = ex->ks.slot_bytes;
    r->blocks = (uint32_t)ex->blocks;
    r->threads = (uint32_t)ex->threads;
    r->table_generation = tag;
    r->table_cleared = clear ? 1 : 0;
    if (graph) {
        // the graph read back the set hash, the table count and the first kGraphLevels level counts
        const uint32_t head = std::min(c.nlevels, kGraphLevels);
        memcpy(r->level_counts, ex->h_levels, sizeof(uint64_t) * head);
        if (c.nlevels > head)
            GPX_CUDA(cudaMemcpy(r->level_counts + head, ex->d_levels + head, sizeof(uint64_t) * (c.nlevels - head),
                                cudaMemcpyDeviceToHost));
        r->set_hash = ex->h_scalar[0];
        r->table_count = ex->h_scalar[1];
        r->d2h_bytes = sizeof(Ctrl) + 16 + (uint64_t)kGraphLevels * 8 +
                       (c.nlevels > head ? (uint64_t)(c.nlevels - head) * 8 : 0);
    } else {
        GPX_CUDA(cudaMemcpyAsync(r->level_counts, ex->d_levels, sizeof(uint64_t) * c.nlevels, cudaMemcpyDeviceToHost,
                                 ex->st));
        // set hash over the visited states (gpx_options.set_hash)
        GPX_CUDA(cudaMemsetAsync(ex->d_scalar, 0, 16, ex->st));
        int blocks = (int)std::min<unsigned long long>((count + 255) / 256, 4096);
        if (ex->o.set_hash)
            ex->ks.set_hash(ex->st, std::max(blocks, 1), ex->d_store, count, nullptr, 0, r->key_words, ex->d_scalar);
        if (ex->o.collect_states || ex->o.verbosity >= 2)
            ex->ks.count(ex->st, count_blocks(ex), ex->d_table, ex->slots, ex->d_ctrl, ex->d_scalar + 1);
        GPX_CUDA(cudaGetLastError());
        unsigned long long h[2] = {0, 0};
        GPX_CUDA(cudaMemcpyAsync(h, ex->d_scalar, 16, cudaMemcpyDeviceToHost, ex->st));
        GPX_CUDA(cudaStreamSynchronize(ex->st));
        r->set_hash = h[0];
        r->table_count = h[1];
        r->h2d_bytes += (launches - 1) * 2 * sizeof(unsigned int); // -k rearm between launches
        r->d2h_bytes = launches * sizeof(Ctrl) + (uint64_t)c.nlevels * 8 + 16;
    }
    if (ex->property == GPX_PROP_LIVENESS && r->status == GPX_OK && r->stopped == GPX_STOP_DONE) {
        // the whole state space is in the table: look for an accepting cycle
        unsigned long long left = 0, rounds = 0;
        GPX_CUDA(cudaEventRecord(ex->ev[0], ex->st));
        int rc = live_check(ex->kind, ex->d_table, ex->nbuckets, ex->slots, ex->d_store, count, ex->d_model,
                            ex->o.seed, ex->st, &ex->live, &left, &rounds);
        if (rc != GPX_OK) return rc;
        GPX_CUDA(cudaEventRecord(ex->ev[1], ex->st));
        GPX_CUDA(cudaEventSynchronize(ex->ev[1]));
        float ms = 0;
        cudaEventElapsedTime(&ms, ex->ev[0], ex->ev[1]);
        r->live_ms = ms;
        r->live_states = left;
        r->live_rounds = rounds;
        if (left) {
            r->verdict = GPX_PROP_LIVENESS;
            r->stopped = GPX_STOP_VIOLATION;
        }
    }
    if (ex->o.collect_states) {
        std::vector<uint32_t> w;
        int rc = collect_words(ex, count, &w);
        if (rc != GPX_OK) return rc;
        r->states_buf = (uint32_t *)malloc(std::max<size_t>(w.size(), 1) * 4);
        memcpy(r->states_buf, w.data(), w.size() * 4);
    }
    ex->last_count = count;
    ex->last_lo = c.lo;
    ex->last_hi = c.hi;
    return r->status;
}

int gpx_explorer_set_por_model(gpx_explorer *ex, const gpx_por_model *m) {
    if (!ex) return GPX_ERR_INVALID;
    if (!m) {
        ex->have_por_model = false;
        return GPX_OK;
    }
    if (!ex->d_por_model) GPX_CUDA(cudaMalloc(&ex->d_por_model, sizeof(gpx_por_model)));
    GPX_CUDA(cudaMemcpy(ex->d_por_model, m, sizeof(gpx_por_model), cudaMemcpyHostToDevice));
    ex->have_por_model = true;
    return GPX_OK;
}

int gpx_explorer_set_por_log(gpx_explorer *ex, uint64_t capacity, uint32_t sample_every) {
    if (!ex) return GPX_ERR_INVALID;
    if (ex->d_log) cudaFree(ex->d_log);
    ex->d_log = nullptr;
    ex->log_cap = 0;
    if (!capacity || !sample_every) return GPX_OK;
    GPX_CUDA(cudaMalloc(&ex->d_log, capacity * sizeof(gpx_por_log_row)));
    if (!ex->d_log_count) GPX_CUDA(cudaMalloc(&ex->d_log_count, 8));
    GPX_CUDA(cudaMemset(ex->d_log_count, 0, 8));
    ex->log_cap = capacity;
    ex->log_every = sample_every;
    return GPX_OK;
}

int gpx_explorer_get_por_log(gpx_explorer *ex, gpx_por_log_row *rows, uint64_t capacity, uint64_t *nrows) {
    if (!ex || !nrows) return GPX_ERR_INVALID;
    *nrows = 0;
    if (!ex->d_log) return GPX_OK;
    unsigned long long n = 0;
    GPX_CUDA(cudaMemcpy(&n, ex->d_log_count, 8, cudaMemcpyDeviceToHost));
    n = std::min<unsigned long long>(n, ex->log_cap);
    *nrows = n;
    if (rows && capacity)
        GPX_CUDA(cudaMemcpy(rows, ex->d_log, std::min<unsigned long long>(n, capacity) * sizeof(gpx_por_log_row),
                            cudaMemcpyDeviceToHost));
    return GPX_OK;
}

int gpx_explore(const gpx_model *model, const gpx_options *opts, gpx_result *result) {
    if (!result) return GPX_ERR_INVALID;
    memset(result, 0, sizeof *result);
    result->struct_size = sizeof *result;
    gpx_explorer *ex = nullptr;
    int rc = gpx_explorer_create(model, opts, &ex);
    if (rc != GPX_OK) {
        result->status = rc;
        result->stopped = GPX_STOP_ERROR;
        return rc;
    }
    rc = gpx_explorer_run(ex, result);
    gpx_explorer_destroy(ex);
    return rc;
}

void gpx_result_free(gpx_result *r) {
    if (!r) return;
    free(r->level_counts);
    free(r->states_buf);
    r->level_counts = nullptr;
    r->states_buf = nullptr;
}

int gpx_explorer_dump(gpx_explorer *ex, const char *path) {
    if (!ex || !path) return GPX_ERR_INVALID;
    FILE *f = fopen(path, "w");
    if (!f) return GPX_ERR_INVALID;
    std::vector<uint32_t> w;
    int rc = collect_words(ex, ex->last_count, &w);
    if (rc == GPX_OK) {
        // the level that would have been expanded next, [lo, count), is unexplored
        unsigned long long unexplored_from = std::min(ex->last_lo, ex->last_count);
        if (ex->h_ctrl->stop == GPX_STOP_DONE) unexplored_from = ex->last_count;
        print_states(f, ex, w, ex->last_count, unexplored_from);
    }
    fclose(f);
    return rc;
}

} // extern "C"

// ======================================================= bounded-wait self-test

namespace gpx {
// Waits with wait_change() on a flag that nothing sets; it must give up.
__global__ void wait_selftest_kernel(const unsigned int *flag, unsigned long long timeout_ns, unsigned int *status,
                                     unsigned long long *waited_ns) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint64_t t0 = globaltimer();
    bool changed = wait_change(flag, 0u, timeout_ns);
    *waited_ns = globaltimer() - t0;
    *status = changed ? GPX_OK : GPX_ERR_TIMEOUT;
}
} // namespace gpx

extern "C" int gpx_selftest_bounded_wait(int device, uint64_t timeout_ns, uint64_t *waited_ns) {
    if (!waited_ns || timeout_ns == 0 || timeout_ns > 10ull * 1000 * 1000 * 1000) return GPX_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GPX_ERR_NO_GPU;
    GPX_CUDA(cudaSetDevice(device));
    unsigned int *d = nullptr;
    GPX_CUDA(cudaMalloc(&d, 64));
    cudaMemset(d, 0, 64);
    wait_selftest_kernel<<<1, 32>>>(d, timeout_ns, d + 1, (unsigned long long *)(d + 2));
    unsigned int h[4] = {0, 0, 0, 0};
    cudaError_t e = cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return GPX_ERR_CUDA;
    *waited_ns = (uint64_t)h[2] | ((uint64_t)h[3] << 32);
    return (int)h[1];
}

// ======================================================= random-access roofline probe

namespace gpx {
// One random 32-byte sector per thread per iteration, read with the hash
// probe's load (ld.global.cg, 256 bits).  The XOR keeps the loads alive.
__global__ void random_gather_kernel(const uint32_t *buf, unsigned long long nsec, int iters,
                                     unsigned long long seed, uint32_t *sink) {
    uint32_t acc = 0;
    unsigned long long tid = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    for (int i = 0; i < iters; i++) {
        unsigned long long s = __umul64hi(mix64(seed ^ (tid * 0x9E3779B97F4A7C15ull + (unsigned)i)), nsec);
        uint32_t w[8];
        ld256_cg(buf + 8 * s, w);
        acc ^= w[0] ^ w[7];
    }
    if (acc == 0x9E3779B9u) sink[0] = acc;
}
} // namespace gpx

// An insert's access: read a random 32-byte bucket, then a 128-bit CAS on its
// first slot against what was read (the sector is dirtied and later written back).
__global__ void random_insert_kernel(uint32_t *buf, unsigned long long nsec, int iters, unsigned long long seed) {
    unsigned long long tid = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    for (int i = 0; i < iters; i++) {
        unsigned long long s = __umul64hi(mix64(seed ^ (tid * 0x9E3779B97F4A7C15ull + (unsigned)i)), nsec);
        uint32_t w[8];
        ld256_cg(buf + 8 * s, w);
        const unsigned long long lo = (unsigned long long)w[0] | ((unsigned long long)w[1] << 32);
        const unsigned long long hi = (unsigned long long)w[2] | ((unsigned long long)w[3] << 32);
        unsigned long long olo, ohi;
        cas128(buf + 8 * s, lo, hi, lo + 1ull, hi, olo, ohi);
    }
}

namespace {

// Random-access rate over a `bytes` buffer: mode 0 gathers 32-byte sectors,
// mode 1 makes insert-like read + CAS accesses.  Best of three timed launches.
int random_access_probe(int device, uint64_t bytes, int mode, double *per_s) {
    if (!per_s || bytes < (1u << 20)) return GPX_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GPX_ERR_NO_GPU;
    GPX_CUDA(cudaSetDevice(device));
    uint32_t *buf = nullptr, *sink = nullptr;
    GPX_CUDA(cudaMalloc(&buf, bytes));
    if (cudaMalloc(&sink, 4) != cudaSuccess) {
        cudaFree(buf);
        return GPX_ERR_NOMEM;
    }
    cudaMemset(buf, 1, bytes);
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, device);
    const int blocks = prop.multiProcessorCount * 8, threads = 256, iters = 256;
    // same L2 fetch hint as the explorer's runs (one sector per miss), restored below
    size_t saved_fetch = 0;
    bool restore = cudaDeviceGetLimit(&saved_fetch, cudaLimitMaxL2FetchGranularity) == cudaSuccess &&
                   cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, 32) == cudaSuccess;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(a);
        if (mode == 0)
            random_gather_kernel<<<blocks, threads>>>(buf, bytes / 32, iters, 0x5851F42D4C957F2Dull + rep, sink);
        else // the dirty sectors of one launch are written back during the next
            random_insert_kernel<<<blocks, threads>>>(buf, bytes / 32, iters, 0x5851F42D4C957F2Dull + rep);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0 && ms < best) best = ms; // the first launch warms up
    }
    cudaError_t e = cudaGetLastError();
    if (restore) cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, saved_fetch);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(buf);
    cudaFree(sink);
    if (e != cudaSuccess) return GPX_ERR_CUDA;
    *per_s = (double)blocks * threads * iters / (best * 1e-3);
    return GPX_OK;
}

} // namespace

extern "C" int gpx_random_insert_probe(int device, uint64_t bytes, double *inserts_per_s) {
    return random_access_probe(device, bytes, 1, inserts_per_s);
}

extern "C" int gpx_random_gather_probe(int device, uint64_t bytes, double *gathers_per_s) {
    return random_access_probe(device, bytes, 0, gathers_per_s);
}


// ======================================================= allocation-free entry point
//
// gpx_explore_noalloc runs the same kernels as gpx_explore with every piece of
// device scratch -- control block, set-hash scalars, level counts, model,
// hash table, state store, cluster array -- carved out of one static device
// array, so the call allocates nothing.  Layout (byte offsets):
//   [0, 1024)           Ctrl (at most 1024 bytes, checked at compile time)
//   [1024, 1088)        set-hash / table-count scalars
//   [4096, +8 MiB)      level counts (kMaxLevels entries)
//   then                model words, hash table, state store, cluster array,
//                       each on a 256-byte boundary
static __device__ __align__(256) unsigned char g_gpx_noalloc_scratch[GPX_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kNoallocMaxDevices = 256;
std::mutex g_noalloc_mutex;
void *g_noalloc_base[kNoallocMaxDevices] = {nullptr};

// Device address of the static array on `device` (current), looked up once per device.
int noalloc_base(int device, unsigned char **out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (device < 0 || device >= kNoallocMaxDevices) return GPX_ERR_INVALID;
    if (!g_noalloc_base[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_gpx_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "gpx_explore_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            return GPX_ERR_CUDA;
        }
        g_noalloc_base[device] = p;
    }
    *out = (unsigned char *)g_noalloc_base[device];
    return GPX_OK;
}

size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

} // namespace

extern "C" int gpx_explore_noalloc(const gpx_model *model, const gpx_options *opts, uint64_t *level_counts,
                                   uint32_t level_capacity, gpx_result *r) {
    if (!model || !r) return GPX_ERR_INVALID;
    if (int bad = check_options(opts)) return bad;
    if (!level_counts && level_capacity) return GPX_ERR_INVALID;
    memset(r, 0, sizeof *r);
    r->struct_size = sizeof *r;
    auto t_start = std::chrono::steady_clock::now();
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GPX_ERR_NO_GPU;
    if (opts->device < 0 || opts->device >= ndev) return GPX_ERR_INVALID;
    GPX_CUDA(cudaSetDevice(opts->device));
    unsigned char *base = nullptr;
    int rc = noalloc_base(opts->device, &base);
    if (rc != GPX_OK) return rc;

    const int mode = opts->por ? (opts->cycle_proviso ? MODE_PROVISO : MODE_POR) : MODE_PLAIN;
    int property = opts->property;
    if (property == GPX_PROP_SAFETY && model->gpf.liveness == 1) property = GPX_PROP_LIVENESS;
    if (property == GPX_PROP_LIVENESS) return GPX_ERR_UNSUPPORTED; // the cycle check needs scratch of its own
    const int kind = select_kind(model->dec.state_bits, false); // the table is cleared on every call
    KernelSet ks = kernels_of(kind);

    // carve the array
    const size_t total = GPX_NOALLOC_SCRATCH_BYTES;
    const size_t off_ctrl = 0, off_scalar = 1024, off_levels = 4096;
    static_assert(sizeof(Ctrl) <= 1024, "the control block must fit below the scalar slot");
    const size_t off_model = round_up(off_levels + (size_t)kMaxLevels * 8, 256);
    const size_t model_bytes = model->dec.words.size() * 4;
    const size_t off_table = round_up(off_model + model_bytes, 256);
    if (off_table >= total) {
        fprintf(stderr, "gpx_explore_noalloc: model of %zu bytes does not fit in the %zu-byte scratch array\n",
                model_bytes, total);
        return GPX_ERR_INVALID;
    }
    const size_t bucket_bytes = (size_t)ks.slot_bytes * ks.bucket_slots;
    const size_t per_state = ks.slot_bytes + (mode == MODE_PROVISO ? 4 : 0);
    size_t left = total - off_table;
    size_t tb = opts->q_words ? (size_t)opts->q_words * 4 : left / 2; // q_words <= 2^60: no wrap
    tb = tb / (2 * bucket_bytes) * (2 * bucket_bytes);
    // the store and the cluster array each start on a 256-byte boundary (512 bytes of slack);
    // sizes are compared in states so that a huge store_states cannot wrap the product
    const size_t max_cap = (tb <= left && left - tb > 512) ? (left - tb - 512) / per_state : 0;
    size_t cap = opts->store_states ? (size_t)opts->store_states : max_cap;
    if (tb < 2 * bucket_bytes || tb > left || cap < 1 || cap > max_cap) {
        fprintf(stderr,
                "gpx_explore_noalloc: requested %zu table bytes + %zu states x %zu bytes, but only %zu bytes of the "
                "%zu-byte scratch array are left after the control block, level counts and model\n",
                tb, cap, per_state, left, total);
        return GPX_ERR_INVALID;
    }
    const size_t off_store = off_table + tb;
    const size_t off_sel = round_up(off_store + cap * ks.slot_bytes, 256);
    if (mode == MODE_PROVISO && off_sel + cap * 4 > total) {
        fprintf(stderr, "gpx_explore_noalloc: the cluster array does not fit in the scratch array\n");
        return GPX_ERR_INVALID;
    }

    // launch shape (no allocation: attributes and occupancy queries only)
    cudaDeviceProp prop;
    GPX_CUDA(cudaGetDeviceProperties(&prop, opts->device));
    int threads = opts->threads > 0 ? opts->threads : 256;
    size_t scratch = (size_t)(threads / 32) * ks.scratch_bytes[mode];
    size_t mb = (model_bytes + 127) & ~(size_t)127;
    bool in_smem = (mb + scratch <= prop.sharedMemPerBlockOptin) && model_bytes <= 96 * 1024;
    size_t smem = scratch + (in_smem ? mb : 0);
    if (smem > prop.sharedMemPerBlockOptin) return GPX_ERR_UNSUPPORTED;
    GPX_CUDA(cudaFuncSetAttribute((const void *)ks.explore[mode], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    int per_sm = 0;
    GPX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)ks.explore[mode], threads, smem));
    if (per_sm < 1) return GPX_ERR_UNSUPPORTED;
    int max_blocks = per_sm * prop.multiProcessorCount;
    int blocks = std::max(1, opts->blocks > 0 ? std::min(opts->blocks, max_blocks) : max_blocks);

    Ctrl *d_ctrl = (Ctrl *)(base + off_ctrl);
    unsigned long long *d_scalar = (unsigned long long *)(base + off_scalar);
    Params P;
    memset(&P, 0, sizeof P);
    P.table = base + off_table;
    P.nbuckets = tb / bucket_bytes;
    P.store = base + off_store;
    P.store_cap = cap;
    P.model = (const uint32_t *)(base + off_model);
    P.model_words = (uint32_t)model->dec.words.size();
    P.model_in_smem = in_smem;
    P.sel = mode == MODE_PROVISO ? (uint32_t *)(base + off_sel) : nullptr;
    P.levels = (unsigned long long *)(base + off_levels);
    P.ctrl = d_ctrl;
    P.seed = opts->seed;
    P.max_states = opts->max_states;
    P.timeout_ns = 20ull * 1000 * 1000 * 1000;
    P.property = (uint32_t)property;
    P.levels_per_launch = opts->kernel_iters > 0 ? (uint32_t)opts->kernel_iters : 0;
    P.total_warps = (uint32_t)(blocks * (threads / 32));
    P.batch_states = batch_states_of(mode, model->dec.nstates.size());
    P.por_kind = por_kind_of(opts->por);

    // clear what must start at zero (the array keeps the previous call's contents;
    // init_kernel resets the control block).  The calling thread's per-thread
    // default stream: no implicit wait on the caller's other blocking streams.
    cudaStream_t st = cudaStreamPerThread;
    Ctrl c;
    GPX_CUDA(cudaMemcpyAsync(base + off_model, model->dec.words.data(), model_bytes, cudaMemcpyHostToDevice, st));
    GPX_CUDA(cudaMemsetAsync(P.table, 0, tb, st));
    GPX_CUDA(cudaMemsetAsync(d_scalar, 0, 64, st));
    ks.init<<<1, 32, 0, st>>>(P, mode == MODE_PROVISO ? PH_DECIDE : PH_EXPAND, 1u);
    GPX_CUDA(cudaGetLastError());
    GPX_CUDA(cudaStreamSynchronize(st));
    auto t_kernels = std::chrono::steady_clock::now();
    void *args[] = {&P};
    unsigned long long launches = 0;
    for (;;) {
        GPX_CUDA(cudaLaunchCooperativeKernel((const void *)ks.explore[mode], dim3(blocks), dim3(threads), args, smem,
                                             st));
        launches++;
        GPX_CUDA(cudaMemcpyAsync(&c, d_ctrl, sizeof c, cudaMemcpyDeviceToHost, st));
        GPX_CUDA(cudaStreamSynchronize(st));
        if (c.done || c.error) break;
        unsigned int zero = 0;
        GPX_CUDA(cudaMemcpyAsync(&d_ctrl->pause, &zero, sizeof zero, cudaMemcpyHostToDevice, st));
        GPX_CUDA(cudaMemcpyAsync(&d_ctrl->launch_levels, &zero, sizeof zero, cudaMemcpyHostToDevice, st));
    }
    auto t_end = std::chrono::steady_clock::now();
    unsigned long long count = std::min<unsigned long long>(c.store_count, cap);
    int hb = (int)std::max<unsigned long long>(1, std::min<unsigned long long>((count + 255) / 256, 4096));
    if (opts->set_hash) ks.set_hash(st, hb, P.store, count, nullptr, 0, model->dec.key_words, d_scalar);
    GPX_CUDA(cudaGetLastError());
    unsigned long long h = 0;
    GPX_CUDA(cudaMemcpyAsync(&h, d_scalar, sizeof h, cudaMemcpyDeviceToHost, st));
    uint32_t ncopy = std::min<uint32_t>(c.nlevels, level_capacity);
    if (ncopy)
        GPX_CUDA(cudaMemcpyAsync(level_counts, P.levels, sizeof(uint64_t) * ncopy, cudaMemcpyDeviceToHost, st));
    GPX_CUDA(cudaStreamSynchronize(st));

    r->status = c.error ? (int)c.error : GPX_OK;
    r->stopped = c.error ? GPX_STOP_ERROR : (int)c.stop;
    r->verdict = (c.stop == GPX_STOP_VIOLATION) ? property : GPX_PROP_NONE;
    r->states = count;
    r->nlevels = c.nlevels;
    r->level_counts = level_counts;
    r->transitions = c.inserts_lookups;
    r->probes = c.probes;
    r->inserts = c.inserts;
    r->lookups = c.lookups;
    r->expanded = c.expanded;
    r->launches = launches;
    r->kernel_ms = std::chrono::duration<double, std::milli>(t_end - t_kernels).count();
    r->explore_ms = r->kernel_ms;
    r->setup_ms = std::chrono::duration<double, std::milli>(t_kernels - t_start).count();
    r->set_hash = h;
    r->key_words = model->dec.key_words;
    r->table_slots = P.nbuckets * ks.bucket_slots;
    r->slot_bytes = ks.slot_bytes;
    r->table_cleared = 1;
    r->blocks = (uint32_t)blocks;
    r->threads = (uint32_t)threads;
    return r->status;
}
