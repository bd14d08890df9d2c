// gpx_live.cu -- liveness: accepting-cycle detection on the explored state space.
//
// The gpf liveness flag (GPUexplore.cu:1888-1898) is parsed by the reference and
// never checked.  Here it means: the last process is a Buchi automaton whose
// local state 1 is accepting, and the property is violated iff a reachable
// cycle passes through an accepting state.  The check runs after a complete
// exploration (no POR) over the state store (a state's identity is its store
// position, found from a successor through its table slot and a slot -> position
// map written once), with the One-Way-Catch-Them-Young fixpoint (Cerna and
// Pelanek, 2003):
//
//   S := visited states
//   repeat
//     S := states of S reachable inside S from accepting states of S
//     S := S without, repeatedly, the states that have no predecessor in S
//   until S does not change
//
// S is empty iff there is no accepting cycle.  Both steps are frontier
// sweeps over the successor relation (the exploration kernels' relation: local
// targets, and for every rule the state's lowest member leads, the product of
// the members' targets).  When memory allows, the relation is built once as
// edge lists of store positions -- one pass that generates every successor and
// finds its slot -- and every sweep then reads lists and per-state flags that
// stay in L2; otherwise each sweep regenerates successors and looks them up.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>

#include "gpx.h"
#include "gpx_device.cuh"
#include "gpx_live.h"
#include "gpx_model.h"

namespace gpx {

constexpr uint32_t kInSet = 1u, kMarked = 2u;

// Slot of a key in a table that no one writes to (the key must be present;
// ~0 otherwise).
template <class K>
__device__ unsigned long long find_slot(const K *table, unsigned long long nb, const K &key, uint64_t h) {
    constexpr int S = KT<K>::kSlots;
    const uint32_t tag = KT<K>::tag_of(key);
    for (int i = 0; i < kMaxProbe; i++) {
        const unsigned long long b = bucket_of(h, i, nb);
        K s[S];
        KT<K>::bucket(const_cast<K *>(table) + b * S, s);
#pragma unroll
        for (int j = 0; j < S; j++) {
            if (KT<K>::eq(s[j], key)) return b * S + j;
            if (KT<K>::empty(s[j], tag)) return ~0ull;
        }
    }
    return ~0ull;
}

// Every successor of `key` under the full transition relation, in the order
// of the oracle's enumeration (processes' local targets, then rules).
template <class K, class F> __device__ void for_each_successor(const MView &M, const K &key, F &&f) {
    const uint32_t n = M.n;
    for (uint32_t p = 0; p < n; p++) {
        uint32_t s;
        const uint32_t *rec = M.state_rec(key, p, s);
        const uint32_t d = M.pd(p);
        for (uint32_t i = 0; i < rec[R_LCNT]; i++) {
            K v = key;
            KT<K>::set(v, MView::fb_of(d), MView::bs_of(d), M.ltgt(rec[R_LOFF] + i));
            f(v);
        }
        for (uint32_t j = 0; j < rec[R_RCNT]; j++) {
            const uint32_t k = M.lrule(rec[R_ROFF] + j);
            const uint32_t mask = M.rmask(k), a = M.ract(k);
            const uint32_t *g[kMaxProcs];
            uint32_t parts[kMaxProcs], idx[kMaxProcs], np = 0;
            bool ok = true;
            for (uint32_t q = 0; q < n && ok; q++) {
                if (!(mask >> q & 1u)) continue;
                uint32_t sq;
                const uint32_t *gq = M.group(M.state_rec(key, q, sq), a);
                if (!gq) {
                    ok = false;
                } else {
                    g[np] = gq;
                    parts[np] = q;
                    idx[np] = 0;
                    np++;
                }
            }
            if (!ok) continue;
            for (;;) {
                K v = key;
                for (uint32_t t = 0; t < np; t++) {
                    const uint32_t dq = M.pd(parts[t]);
                    KT<K>::set(v, MView::fb_of(dq), MView::bs_of(dq), M.stgt(g[t][1] + idx[t]));
                }
                f(v);
                uint32_t t = 0;
                while (t < np && ++idx[t] == g[t][2]) idx[t++] = 0;
                if (t == np) break;
            }
        }
    }
}

__device__ __forceinline__ void push(uint32_t *front, unsigned long long *n, unsigned long long cap, uint32_t i,
                                     unsigned long long *overflow) {
    const unsigned long long k = atomicAdd(n, 1ull);
    if (k < cap)
        front[k] = i;
    else
        atomicAdd(overflow, 1ull);
}

// Store position of a successor (~0u when it is missing from the table).
template <class K>
__device__ __forceinline__ uint32_t position_of(const K *table, unsigned long long nb, const uint32_t *index,
                                                const K &v, unsigned long long seed) {
    const unsigned long long j = find_slot(table, nb, v, KT<K>::hash(v, seed));
    return j == ~0ull ? ~0u : __ldg(index + j);
}

// count[0]: |S|, count[1]: frontier size, count[2]: next frontier size, count[3]: overflow / missing states,
// count[4]: edges of the successor lists

// Successors of the state at store position i, as store positions: read from
// the edge lists when they were built (edges != null), else regenerated and
// looked up in the table.
template <class K> struct Succ {
    const K *table;
    unsigned long long nb;
    const uint32_t *index;
    const K *store;
    unsigned long long seed;
    const unsigned long long *beg;
    const uint32_t *deg;
    const uint32_t *edges;
    template <class F> __device__ void each(const MView &M, uint32_t i, F &&f) const {
        if (edges) {
            const unsigned long long b = beg[i];
            const uint32_t d = deg[i];
            for (uint32_t k = 0; k < d; k++) f(__ldg(edges + b + k));
            return;
        }
        const K key = KT<K>::load(store + i);
        for_each_successor(M, key, [&](const K &v) { f(position_of(table, nb, index, v, seed)); });
    }
};

// Out-degree of every state and the start of its edge list (one atomic per warp).
template <class K>
__global__ void live_degree_kernel(const K *store, unsigned long long states, const uint32_t *model, uint32_t *deg,
                                   unsigned long long *beg, unsigned long long *count) {
    MView M;
    M.init(model);
    const uint32_t lane = threadIdx.x & 31;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i0 = blockIdx.x * (unsigned long long)blockDim.x + (threadIdx.x & ~31u); i0 < states;
         i0 += stride) {
        const unsigned long long i = i0 + lane;
        uint32_t c = 0;
        if (i < states) {
            for_each_successor(M, KT<K>::load(store + i), [&](const K &) { c++; });
            deg[i] = c;
        }
        unsigned long long incl = c;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(kFull, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        unsigned long long base = 0;
        if (lane == 31) base = atomicAdd(&count[4], incl);
        base = __shfl_sync(kFull, base, 31);
        if (i < states) beg[i] = base + incl - c;
    }
}

// The edge lists: every successor's store position.
template <class K>
__global__ void live_fill_kernel(const K *table, unsigned long long nb, const uint32_t *index, const K *store,
                                 unsigned long long states, const uint32_t *model, unsigned long long seed,
                                 const unsigned long long *beg, uint32_t *edges, unsigned long long *count) {
    MView M;
    M.init(model);
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < states;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        unsigned long long e = beg[i];
        for_each_successor(M, KT<K>::load(store + i), [&](const K &v) {
            const uint32_t j = position_of(table, nb, index, v, seed);
            if (j == ~0u) atomicAdd(&count[3], 1ull);
            edges[e++] = j;
        });
    }
}

// The slot -> store position map, and S := every state.
template <class K>
__global__ void live_init_kernel(const K *table, unsigned long long nb, const K *store, unsigned long long states,
                                 unsigned long long seed, uint32_t *index, uint32_t *flag, uint32_t *indeg,
                                 unsigned long long *count) {
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < states;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const K key = KT<K>::load(store + i);
        const unsigned long long j = find_slot(table, nb, key, KT<K>::hash(key, seed));
        if (j == ~0ull)
            atomicAdd(&count[3], 1ull);
        else
            index[j] = (uint32_t)i;
        flag[i] = kInSet;
        indeg[i] = 0;
    }
}

// Mark the accepting states of S and put them in the frontier.
template <class K>
__global__ void live_seed_kernel(const K *store, unsigned long long states, const uint32_t *model, uint32_t *flag,
                                 uint32_t *front, unsigned long long cap, unsigned long long *count) {
    MView M;
    M.init(model);
    const uint32_t d = M.pd(M.n - 1);
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < states;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        if (!(flag[i] & kInSet)) continue;
        if (KT<K>::get(KT<K>::load(store + i), MView::fb_of(d), MView::bs_of(d)) != 1) continue;
        flag[i] |= kMarked;
        push(front, &count[1], cap, (uint32_t)i, &count[3]);
    }
}

// One forward round: mark the unmarked successors in S of the frontier.
template <class K>
__global__ void live_reach_kernel(Succ<K> S, const uint32_t *model, uint32_t *flag, const uint32_t *front,
                                  unsigned long long nfront, uint32_t *next, unsigned long long cap,
                                  unsigned long long *count) {
    MView M;
    M.init(model);
    for (unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; t < nfront;
         t += (unsigned long long)gridDim.x * blockDim.x) {
        S.each(M, front[t], [&](uint32_t j) {
            if (j == ~0u) {
                atomicAdd(&count[3], 1ull);
                return;
            }
            if ((flag[j] & kInSet) && !(atomicOr(&flag[j], kMarked) & kMarked)) push(next, &count[2], cap, j, &count[3]);
        });
    }
}

// S := marked states of S; clears the marks and the predecessor counts; counts |S|.
__global__ void live_restrict_kernel(unsigned long long states, uint32_t *flag, uint32_t *indeg,
                                     unsigned long long *count) {
    unsigned long long acc = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < states;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t f = flag[i];
        const uint32_t keep = (f & kInSet) && (f & kMarked) ? kInSet : 0u;
        flag[i] = keep;
        indeg[i] = 0;
        acc += keep;
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(&count[0], acc);
}

// Predecessor counts inside S (edges counted with multiplicity).
template <class K>
__global__ void live_indeg_kernel(Succ<K> S, unsigned long long states, const uint32_t *model, const uint32_t *flag,
                                  uint32_t *indeg, unsigned long long *count) {
    MView M;
    M.init(model);
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < states;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        if (!(flag[i] & kInSet)) continue;
        S.each(M, (uint32_t)i, [&](uint32_t j) {
            if (j == ~0u) {
                atomicAdd(&count[3], 1ull);
                return;
            }
            if (flag[j] & kInSet) atomicAdd(&indeg[j], 1u);
        });
    }
}

// The states of S without predecessors in S start the peeling.
__global__ void live_sources_kernel(unsigned long long states, const uint32_t *flag, const uint32_t *indeg,
                                    uint32_t *front, unsigned long long cap, unsigned long long *count) {
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < states;
         i += (unsigned long long)gridDim.x * blockDim.x)
        if ((flag[i] & kInSet) && indeg[i] == 0) push(front, &count[1], cap, (uint32_t)i, &count[3]);
}

// One peeling round: remove the frontier from S; successors whose last
// predecessor in S went form the next frontier.
template <class K>
__global__ void live_peel_kernel(Succ<K> S, const uint32_t *model, uint32_t *flag, uint32_t *indeg,
                                 const uint32_t *front, unsigned long long nfront, uint32_t *next,
                                 unsigned long long cap, unsigned long long *count) {
    MView M;
    M.init(model);
    for (unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; t < nfront;
         t += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t i = front[t];
        flag[i] = 0;
        S.each(M, i, [&](uint32_t j) {
            if (j == ~0u) {
                atomicAdd(&count[3], 1ull);
                return;
            }
            if ((flag[j] & kInSet) && atomicSub(&indeg[j], 1u) == 1u) push(next, &count[2], cap, j, &count[3]);
        });
    }
}

__global__ void live_count_kernel(unsigned long long states, const uint32_t *flag, unsigned long long *count) {
    unsigned long long acc = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < states;
         i += (unsigned long long)gridDim.x * blockDim.x)
        acc += flag[i] & kInSet;
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(&count[0], acc);
}

void live_free(LiveScratch *s) {
    cudaFree(s->index);
    cudaFree(s->flag);
    cudaFree(s->indeg);
    cudaFree(s->deg);
    cudaFree(s->beg);
    cudaFree(s->edges);
    cudaFree(s->front[0]);
    cudaFree(s->front[1]);
    cudaFree(s->count);
    *s = LiveScratch();
}

namespace {

#define LCUDA(call)                                                                                           \
    do {                                                                                                      \
        cudaError_t _e = (call);                                                                              \
        if (_e != cudaSuccess) {                                                                              \
            fprintf(stderr, "gpx liveness: %s failed: %s\n", #call, cudaGetErrorString(_e));               \
            return (_e == cudaErrorMemoryAllocation) ? GPX_ERR_NOMEM : GPX_ERR_CUDA;                          \
        }                                                                                                     \
    } while (0)

int grid_for(unsigned long long n) {
    unsigned long long b = (n + 255) / 256;
    return (int)(b < 1 ? 1 : (b > 8192 ? 8192 : b));
}

template <class K>
int run(const K *table, unsigned long long nb, unsigned long long slots, const K *store, unsigned long long states,
        const uint32_t *model, unsigned long long seed, cudaStream_t st, LiveScratch *s,
        unsigned long long *set_states, unsigned long long *rounds) {
    if (states >= 0xFFFFFFFFull) return GPX_ERR_UNSUPPORTED; // store positions are 32-bit
    if (s->slots < slots) {
        cudaFree(s->index);
        s->index = nullptr;
        LCUDA(cudaMalloc(&s->index, slots * 4));
        s->slots = slots;
    }
    if (s->states < states) {
        for (uint32_t **a : {&s->flag, &s->indeg, &s->front[0], &s->front[1]}) {
            cudaFree(*a);
            *a = nullptr;
            LCUDA(cudaMalloc(a, states * 4));
        }
        s->states = states;
    }
    if (!s->count) LCUDA(cudaMalloc(&s->count, 8 * 8));
    unsigned long long h[5];
    auto read = [&]() -> int {
        LCUDA(cudaMemcpyAsync(h, s->count, sizeof h, cudaMemcpyDeviceToHost, st));
        LCUDA(cudaStreamSynchronize(st));
        if (h[3]) {
            fprintf(stderr, "gpx liveness: %llu successors missing from the table or frontier overflow\n", h[3]);
            return GPX_ERR_INVALID;
        }
        return GPX_OK;
    };
    const unsigned long long cap = s->states;
    const int gs = grid_for(states);
    *rounds = 0;
    LCUDA(cudaMemsetAsync(s->count, 0, sizeof h, st));
    live_init_kernel<K><<<gs, 256, 0, st>>>(table, nb, store, states, seed, s->index, s->flag, s->indeg, s->count);
    LCUDA(cudaGetLastError());
    int rc = read();
    if (rc) return rc;
    // the successor relation as edge lists of store positions, when it fits in
    // half of the free memory; otherwise the sweeps regenerate successors
    Succ<K> S{table, nb, s->index, store, seed, nullptr, nullptr, nullptr};
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && states * 12 < free_b / 4) {
        if (s->lists_cap < states) {
            cudaFree(s->deg);
            cudaFree(s->beg);
            s->deg = nullptr;
            s->beg = nullptr;
            s->lists_cap = 0;
            LCUDA(cudaMalloc(&s->deg, states * 4));
            LCUDA(cudaMalloc(&s->beg, states * 8));
            s->lists_cap = states;
        }
        LCUDA(cudaMemsetAsync(s->count, 0, sizeof h, st));
        live_degree_kernel<K><<<gs, 256, 0, st>>>(store, states, model, s->deg, s->beg, s->count);
        LCUDA(cudaGetLastError());
        if ((rc = read())) return rc;
        const unsigned long long nedges = h[4];
        cudaMemGetInfo(&free_b, &total_b);
        if (s->edges_cap >= nedges || nedges * 4 < free_b / 2) {
            if (s->edges_cap < nedges) {
                cudaFree(s->edges);
                s->edges = nullptr;
                s->edges_cap = 0;
                LCUDA(cudaMalloc(&s->edges, std::max<unsigned long long>(nedges, 1) * 4));
                s->edges_cap = nedges;
            }
            live_fill_kernel<K><<<gs, 256, 0, st>>>(table, nb, s->index, store, states, model, seed, s->beg,
                                                    s->edges, s->count);
            LCUDA(cudaGetLastError());
            if ((rc = read())) return rc;
            S.beg = s->beg;
            S.deg = s->deg;
            S.edges = s->edges;
        }
    }
    unsigned long long size = states;
    for (;;) {
        const unsigned long long before = size;
        // forward closure from the accepting states of S
        LCUDA(cudaMemsetAsync(s->count, 0, sizeof h, st));
        live_seed_kernel<K><<<gs, 256, 0, st>>>(store, states, model, s->flag, s->front[0], cap, s->count);
        LCUDA(cudaGetLastError());
        if ((rc = read())) return rc;
        int cur = 0;
        unsigned long long nfront = h[1];
        while (nfront) {
            LCUDA(cudaMemsetAsync(s->count + 2, 0, 8, st));
            live_reach_kernel<K><<<grid_for(nfront), 256, 0, st>>>(S, model, s->flag, s->front[cur], nfront,
                                                                   s->front[cur ^ 1], cap, s->count);
            LCUDA(cudaGetLastError());
            if ((rc = read())) return rc;
            nfront = h[2];
            cur ^= 1;
            ++*rounds;
        }
        LCUDA(cudaMemsetAsync(s->count, 0, sizeof h, st));
        live_restrict_kernel<<<gs, 256, 0, st>>>(states, s->flag, s->indeg, s->count);
        LCUDA(cudaGetLastError());
        if ((rc = read())) return rc;
        size = h[0];
        if (size == 0) break;
        // peel the states with no predecessor in S
        LCUDA(cudaMemsetAsync(s->count, 0, sizeof h, st));
        live_indeg_kernel<K><<<gs, 256, 0, st>>>(S, states, model, s->flag, s->indeg, s->count);
        LCUDA(cudaGetLastError());
        live_sources_kernel<<<gs, 256, 0, st>>>(states, s->flag, s->indeg, s->front[0], cap, s->count);
        LCUDA(cudaGetLastError());
        if ((rc = read())) return rc;
        cur = 0;
        nfront = h[1];
        while (nfront) {
            LCUDA(cudaMemsetAsync(s->count + 2, 0, 8, st));
            live_peel_kernel<K><<<grid_for(nfront), 256, 0, st>>>(S, model, s->flag, s->indeg, s->front[cur],
                                                                  nfront, s->front[cur ^ 1], cap, s->count);
            LCUDA(cudaGetLastError());
            if ((rc = read())) return rc;
            nfront = h[2];
            cur ^= 1;
            ++*rounds;
        }
        LCUDA(cudaMemsetAsync(s->count, 0, sizeof h, st));
        live_count_kernel<<<gs, 256, 0, st>>>(states, s->flag, s->count);
        LCUDA(cudaGetLastError());
        if ((rc = read())) return rc;
        size = h[0];
        if (size == 0 || size == before) break;
    }
    *set_states = size;
    return GPX_OK;
}

} // namespace

int live_check(int kind, void *table, unsigned long long nbuckets, unsigned long long slots, const void *store,
               unsigned long long states, const uint32_t *model, unsigned long long seed, cudaStream_t st,
               LiveScratch *s, unsigned long long *set_states, unsigned long long *rounds) {
    if (kind == 0)
        return run<K32>((const K32 *)table, nbuckets, slots, (const K32 *)store, states, model, seed, st, s,
                        set_states, rounds);
    if (kind == 1)
        return run<K64>((const K64 *)table, nbuckets, slots, (const K64 *)store, states, model, seed, st, s,
                        set_states, rounds);
    if (kind == 2)
        return run<K128>((const K128 *)table, nbuckets, slots, (const K128 *)store, states, model, seed, st, s,
                         set_states, rounds);
    return run<K128G>((const K128G *)table, nbuckets, slots, (const K128G *)store, states, model, seed, st, s,
                      set_states, rounds);
}

} // namespace gpx
