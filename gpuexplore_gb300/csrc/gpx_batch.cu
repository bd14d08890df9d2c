// gpx_batch.cu -- many gpf networks explored in one persistent launch.
//
// Every instance keeps the single-network semantics (level-synchronous BFS,
// verdicts, budget, cluster POR) but instances advance independently: an
// instance's current level (or POR decide/insert phase) is an "epoch" published
// in a 64-bit ticket (epoch << 40 | claim cursor).  Warps roam over the
// instances, claim chunks of the published level with one atomicAdd on the
// ticket, expand them with the same per-warp engine as the single-network
// kernel (Explorer in gpx_device.cuh), and report the states they completed;
// the warp that completes the last chunk of a level closes it and publishes the
// next epoch.  No grid-wide barrier is needed, so small instances finish and
// free the GPU for large ones.  Each instance has the slot width its state
// vector needs (32, 64 or 128 bits), so a small network's partition holds two
// or four times the states of a 128-bit one in the same bytes.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "gpx.h"
#include "gpx_model.h"
#include "gpx_device.cuh"

namespace gpx {

constexpr unsigned long long kCurMask = (1ull << 40) - 1;
constexpr uint32_t kBatchLevels = 4096;

struct BLevel {
    unsigned long long lo, hi;
    unsigned int phase, pad;
};

struct __align__(128) BInst {
    Ctrl ctrl;                      // counters, status, stop reason, done flag, level count
    // The ticket (polled by scanning warps, an atomic per claim), the completion
    // counters (an atomic per claim) and the levels (read with every ticket) on
    // lines of their own: sharing one line cost the ten config-1 rings in one
    // batch 1.17 instead of 0.84 ms, config 5 430 instead of 386 ms.
    alignas(128) unsigned long long ticket; // epoch << 40 | cursor
    alignas(128) unsigned long long completed[2];
    alignas(128) BLevel lvl[2];     // the level of each epoch parity
    unsigned long long finish_ns;
    // set up by the host
    void *table;                    // slots of the instance's width (kind)
    unsigned long long nbuckets;
    void *store;
    unsigned long long store_cap;
    const uint32_t *model;
    uint32_t *aux;                  // per store position: the cluster (cycle proviso) or the
                                    // inserting move's participants (plain, pruning); else null
    unsigned long long *levels;
    unsigned long long max_states;
    uint32_t property, mode;
    uint32_t por_kind;              // POR_CAMPLE / POR_AMPLE / POR_STUBBORN (job por 1-2 / 3 / 4)
    uint32_t kind;                  // slot width: 0 = 32, 1 = 64, 2 = 128 bits
    const gpx_por_model *por_model; // learned proposal (job por == 2), else null
    void *overflow;                 // keys whose probe sequence was full during the current level,
    unsigned long long overflow_cap; // placed with eviction by the warp that closes it
};

struct BGlobal {
    unsigned int done_count;
    unsigned int error;
    unsigned long long start_ns;
    unsigned long long launches; // batch_kernel launches of this admission round
};

constexpr unsigned long long kMaxBatchLaunches = 1ull << 24;

struct BParams {
    BInst *inst;
    BGlobal *g;
    uint32_t count;
    uint32_t claim;
    uint32_t max_claims;
    uint32_t total_warps;
    uint32_t latency_sms; // SMs [0, latency_sms) serve only latency-critical phases
    unsigned long long seed;
    unsigned long long timeout_ns;
};

// A phase is latency-critical when it is small and its instance is deep: such
// instances advance one short phase at a time, and each claim's latency on a
// fully loaded SM (several times that on an idle one) is what bounds them.
constexpr unsigned long long kCriticalStates = 8192;
constexpr unsigned int kCriticalEpochs = 32;

// Acquire load of a ticket: the level it names is read after it.
static __device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

static __device__ BLevel read_level(const BInst *I, unsigned int e) {
    const volatile BLevel *L = &I->lvl[e & 1];
    BLevel r;
    r.lo = L->lo;
    r.hi = L->hi;
    r.phase = L->phase;
    r.pad = 0;
    return r;
}

// Close epoch e of instance I (called by the thread that completed its last chunk).
static __device__ void close_instance(const BParams &BP, BInst *I, unsigned int e) {
    __threadfence();
    BLevel L = read_level(I, e);
    Ctrl *c = &I->ctrl;
    BLevel next;
    next.pad = 0;
    if (I->mode == MODE_PROVISO && L.phase == PH_DECIDE) {
        next.lo = L.lo;
        next.hi = L.hi;
        next.phase = PH_EXPAND;
    } else {
        unsigned long long newhi = vload(&c->store_count);
        if (newhi > I->store_cap) newhi = I->store_cap;
        unsigned long long cnt = newhi - L.hi;
        if (cnt) {
            if (c->nlevels < kBatchLevels)
                I->levels[c->nlevels++] = cnt;
            else
                set_error(c, GPX_ERR_UNSUPPORTED);
        }
        c->level++;
        unsigned int stop = 0xFFFFFFFFu;
        if (vload(&c->error))
            stop = GPX_STOP_ERROR;
        else if (vload(&c->violation))
            stop = GPX_STOP_VIOLATION;
        else if (cnt == 0)
            stop = GPX_STOP_DONE;
        else if (I->max_states && newhi >= I->max_states)
            stop = GPX_STOP_BUDGET;
        if (stop != 0xFFFFFFFFu) {
            c->stop = stop;
            c->lo = L.hi;
            c->hi = newhi;
            I->finish_ns = globaltimer();
            __threadfence();
            c->done = 1;
            atomicAdd(&BP.g->done_count, 1u);
            return;
        }
        next.lo = L.hi;
        next.hi = newhi;
        next.phase = I->mode == MODE_PROVISO ? PH_DECIDE : PH_EXPAND;
    }
    volatile BLevel *N = &I->lvl[(e + 1) & 1];
    N->lo = next.lo;
    N->hi = next.hi;
    N->phase = next.phase;
    I->completed[(e + 1) & 1] = 0;
    __threadfence();
    atomicExch(&I->ticket, (unsigned long long)(e + 1) << 40);
}

// Not inlined: each (slot width, mode) path gets its own register allocation.
template <class K, int MODE>
static __device__ __noinline__ void process_claim(const BParams &BP, BInst *I, unsigned char *raw, unsigned long long lo,
                                     unsigned long long off, unsigned long long cnt, unsigned long long claim,
                                     bool decide) {
    Params P;
    memset(&P, 0, sizeof P);
    P.table = I->table;
    P.nbuckets = I->nbuckets;
    P.store = I->store;
    P.store_cap = I->store_cap;
    P.overflow = I->overflow;
    P.overflow_cap = I->overflow_cap;
    P.model = I->model;
    P.sel = I->mode == MODE_PROVISO ? I->aux : nullptr;
    P.label = I->mode == MODE_PLAIN ? I->aux : nullptr;
    P.ctrl = &I->ctrl;
    P.seed = BP.seed;
    P.timeout_ns = BP.timeout_ns;
    P.property = I->property;
    P.por_model = I->por_model;
    P.learned = I->por_model ? 1u : 0u;
    P.por_kind = I->por_kind;
    // claims of a few states: not the explore kernel's wide-batch machinery
    Explorer<K, MODE, false> E(P, I->model, *(WarpScratch<K, MODE> *)raw);
    uint32_t B = WarpScratch<K, MODE>::kPairs / E.M.n;
    B = B > 32 ? 32 : (B < 1 ? 1 : B);
    if (B > claim) B = (uint32_t)claim; // small claims: one batch per claim, spread over warps
    for (unsigned long long b = off; b < off + cnt; b += B) {
        uint32_t n = (uint32_t)((off + cnt - b) < B ? (off + cnt - b) : B);
        unsigned long long left = off + cnt - b - n;
        E.batch(lo + b, n, b, decide, (uint32_t)(left < B ? left : B));
    }
    E.flush_stats(); // appends the staged new states before the chunk is reported
}

// A claim of instance I with its slot width and mode.
template <class K>
static __device__ void run_claim(const BParams &BP, BInst *I, unsigned char *raw, unsigned long long lo,
                                 unsigned long long off, unsigned long long cnt, unsigned long long claim, bool decide) {
    if (I->mode == MODE_PLAIN)
        process_claim<K, MODE_PLAIN>(BP, I, raw, lo, off, cnt, claim, false);
    else if (I->mode == MODE_POR)
        process_claim<K, MODE_POR>(BP, I, raw, lo, off, cnt, claim, false);
    else
        process_claim<K, MODE_PROVISO>(BP, I, raw, lo, off, cnt, claim, decide);
}

// The level's overflowed keys of instance I, placed by the closing warp.
template <class K> static __device__ __noinline__ void place_instance(const BParams &BP, BInst *I, unsigned long long over,
                                                         uint32_t lane) {
    place_list_warp<K>((K *)I->table, I->nbuckets, (K *)I->store, I->mode == MODE_PLAIN ? I->aux : nullptr,
                       I->store_cap, (const K *)I->overflow, over, &I->ctrl, BP.seed, lane);
}

__global__ void __launch_bounds__(256, 3) batch_kernel(BParams BP) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char *raw = smem + (size_t)(threadIdx.x >> 5) * sizeof(WarpScratch<K128, MODE_PROVISO>);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    // on a reserved SM every resident warp serves latency-critical phases first,
    // other phases only when no critical one is claimable; elsewhere warps leave
    // critical phases to the reserved SMs
    const bool express = smid < BP.latency_sms;
    uint32_t next = gwarp % BP.count;
    uint32_t claims = 0;
    uint64_t idle_since = 0;
    unsigned int idle_ns = 256;
    for (;;) {
        if (vload(&BP.g->done_count) >= BP.count || vload(&BP.g->error)) break;
        if (BP.max_claims && claims >= BP.max_claims) break;
        bool worked = false;
        // The lanes scan 32 instances at a time for a claimable phase (a reserved
        // SM's warp scans the virtual range twice: critical phases only, then any),
        // then the warp tries the candidates in scan order.  A serial scan with a
        // fence per instance took a millisecond over 512 instances.
        const uint32_t span = express ? 2 * BP.count : BP.count;
        for (uint32_t k0 = 0; k0 < span && !worked; k0 += 32) {
            const uint32_t k = k0 + lane;
            uint32_t i = 0;
            bool cand = false;
            if (k < span) {
                const bool any = k >= BP.count;
                i = next + (any ? k - BP.count : k);
                if (i >= BP.count) i -= BP.count;
                const BInst *Ic = &BP.inst[i];
                if (!vload(&Ic->ctrl.done)) {
                    const unsigned long long t = ld_acquire64(&Ic->ticket);
                    const unsigned int e = (unsigned int)(t >> 40);
                    const BLevel Lc = read_level(Ic, e);
                    const unsigned long long n = Lc.hi - Lc.lo;
                    cand = (t & kCurMask) < n;
                    if (cand && BP.latency_sms) {
                        const bool critical = n <= kCriticalStates && e >= kCriticalEpochs;
                        if (express ? (!critical && !any) : critical) cand = false;
                    }
                }
            }
            uint32_t m = __ballot_sync(kFull, cand);
            while (m && !worked) {
                const int src = __ffs(m) - 1;
                m &= m - 1;
                const uint32_t ci = __shfl_sync(kFull, i, src); // this candidate (i stays per lane)
                BInst *I = &BP.inst[ci];
                unsigned long long t = ld_acquire64(&I->ticket);
                unsigned int e = (unsigned int)(t >> 40);
                BLevel L = read_level(I, e);
                unsigned long long n = L.hi - L.lo;
                if ((t & kCurMask) >= n) continue;
                // level-sized claims (at least the tuned size) keep few-state levels on many warps
                unsigned long long claim = n / ((unsigned long long)BP.total_warps * 4ull);
                claim = claim < BP.claim ? BP.claim : (claim > 4096 ? 4096 : claim);
                unsigned long long old = 0;
                if (lane == 0) old = atomicAdd(&I->ticket, claim);
                old = __shfl_sync(kFull, old, 0);
                unsigned int e2 = (unsigned int)(old >> 40);
                unsigned long long cur = old & kCurMask;
                if (e2 != e) {
                    __threadfence();
                    L = read_level(I, e2);
                    n = L.hi - L.lo;
                }
                if (cur >= n) continue;
                unsigned long long cnt = (n - cur) < claim ? (n - cur) : claim;
                bool decide = L.phase == PH_DECIDE;
                if (I->kind == 0)
                    run_claim<K32>(BP, I, raw, L.lo, cur, cnt, claim, decide);
                else if (I->kind == 1)
                    run_claim<K64>(BP, I, raw, L.lo, cur, cnt, claim, decide);
                else
                    run_claim<K128>(BP, I, raw, L.lo, cur, cnt, claim, decide);
                __threadfence();
                unsigned long long d = 0;
                if (lane == 0) d = atomicAdd(&I->completed[e2 & 1], cnt) + cnt;
                if (__shfl_sync(kFull, d, 0) == n) {
                    // every chunk of the epoch is done: the instance is quiescent.  Keys
                    // whose probe sequence was full are placed with eviction first.
                    __threadfence();
                    Ctrl *c = &I->ctrl;
                    const unsigned long long over = vload(&c->overflow_count);
                    if (over) {
                        if (over <= I->overflow_cap && !vload(&c->error)) {
                            if (I->kind == 0)
                                place_instance<K32>(BP, I, over, lane);
                            else if (I->kind == 1)
                                place_instance<K64>(BP, I, over, lane);
                            else
                                place_instance<K128>(BP, I, over, lane);
                        } else if (lane == 0)
                            set_error(c, GPX_ERR_TABLE_FULL); // re-admitted with a larger partition
                        if (lane == 0) c->overflow_count = 0;
                        __threadfence();
                    }
                    if (lane == 0) close_instance(BP, I, e2);
                }
                __syncwarp();
                worked = true;
                next = ci;
                claims++;
            }
        }
        if (worked) {
            idle_since = 0;
            idle_ns = 256;
        } else {
            // nothing claimable right now: other warps are finishing levels.  The
            // sleep doubles up to 8 us, so that thousands of idle warps do not
            // keep polling the few tickets the busy ones claim from (ten rings
            // in one batch: 1.51 -> 1.18 ms)
            __nanosleep(idle_ns);
            if (idle_ns < 8192) idle_ns <<= 1;
            uint64_t now = globaltimer();
            if (!idle_since)
                idle_since = now;
            else if (now - idle_since > BP.timeout_ns) {
                if (lane == 0) atomicCAS(&BP.g->error, 0u, (unsigned int)GPX_ERR_TIMEOUT);
                break;
            }
        }
    }
}

// After each batch_kernel launch of the captured loop: another launch follows
// while instances remain and no error was recorded (each launch makes progress:
// every warp claims until its claim budget is spent or nothing is left).
__global__ void batch_relaunch_kernel(BGlobal *g, uint32_t count, cudaGraphConditionalHandle loop) {
    unsigned int more = g->done_count < count && !g->error;
    g->launches++;
    if (more && g->launches >= kMaxBatchLaunches) {
        atomicCAS(&g->error, 0u, (unsigned int)GPX_ERR_UNSUPPORTED);
        more = 0;
    }
    __threadfence();
    cudaGraphSetConditional(loop, more);
}

template <class K> static __device__ void insert_initial(BInst *I, unsigned long long seed) {
    const K key = KT<K>::initial(0);
    unsigned int probes = 0;
    find_or_insert<K>((K *)I->table, I->nbuckets, key, KT<K>::hash(key, seed), probes);
    ((K *)I->store)[0] = key;
}

// Initial state of every instance (GPUexplore.cu:668-682) and the launch clock.
__global__ void batch_init_kernel(BParams BP, int first_launch) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && first_launch) BP.g->start_ns = globaltimer();
    if (i >= BP.count) return;
    BInst *I = &BP.inst[i];
    if (I->kind == 0)
        insert_initial<K32>(I, BP.seed);
    else if (I->kind == 1)
        insert_initial<K64>(I, BP.seed);
    else
        insert_initial<K128>(I, BP.seed);
    if (I->mode == MODE_PLAIN && I->aux) I->aux[0] = 0; // the initial state's label: nothing pruned
    I->levels[0] = 1;
}

// Per-instance order-independent set hash over each store.
__global__ void batch_hash_kernel(const BInst *inst, uint32_t count, const uint32_t *words,
                                  unsigned long long *out) {
    for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
        const BInst *I = &inst[i];
        unsigned long long cnt = I->ctrl.store_count < I->store_cap ? I->ctrl.store_count : I->store_cap;
        unsigned long long acc = 0;
        for (unsigned long long j = threadIdx.x; j < cnt; j += blockDim.x) {
            uint32_t w[4];
            if (I->kind == 0)
                KT<K32>::words(KT<K32>::load((const K32 *)I->store + j), w);
            else if (I->kind == 1)
                KT<K64>::words(KT<K64>::load((const K64 *)I->store + j), w);
            else
                KT<K128>::words(KT<K128>::load((const K128 *)I->store + j), w);
            uint64_t h = 0x9E3779B97F4A7C15ull;
            for (uint32_t k = 0; k < words[i]; k += 2) {
                uint64_t cc = w[k];
                if (k + 1 < words[i]) cc |= (uint64_t)w[k + 1] << 32;
                h = mix64(h ^ cc);
            }
            acc += h;
        }
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&out[i], acc);
    }
}

} // namespace gpx

using namespace gpx;

namespace {

#define BCUDA(call)                                                                                           \
    do {                                                                                                      \
        cudaError_t _e = (call);                                                                              \
        if (_e != cudaSuccess) {                                                                              \
            fprintf(stderr, "gpx batch: %s failed: %s\n", #call, cudaGetErrorString(_e));                   \
            rc = (_e == cudaErrorMemoryAllocation) ? GPX_ERR_NOMEM : GPX_ERR_CUDA;                            \
            goto done;                                                                                        \
        }                                                                                                     \
    } while (0)

struct BatchConfig {
    int blocks, threads, claim, kernel_iters, latency_sms;
    bool prune_commuting;
    bool narrow_slots; // each instance in the narrowest slot its vector fits (else 128-bit slots for all)
    double load_factor;
};

struct Outcome {
    int status, stopped, verdict;
    uint32_t nlevels;
    uint64_t states, set_hash, capacity;
    double completion_ms;
    std::vector<uint64_t> levels;
};

constexpr unsigned long long kInstOverflow = 1024; // overflowed keys an instance can place per level
constexpr uint32_t kSlotBytes[3] = {4, 8, 16};

// Slot width of an instance: with narrow slots the narrowest that holds its
// state vector and the occupancy bit of each 32/64-bit half (as in a
// single-network table), else 128 bits.  Narrow slots hold two to four times
// the states per byte; 128-bit slots (two per bucket) measured faster on the
// config-5 batch (432 vs 470 ms, p50 15 vs 27 ms): a small instance's 8-slot
// buckets put more concurrent inserts on each sector.
uint32_t slot_kind(const gpx_model *m, bool narrow) {
    const uint32_t bits = m->dec.state_bits;
    if (!narrow) return 2u;
    return bits <= 31 ? 0u : (bits <= 63 ? 1u : 2u);
}

// Device bytes per admitted state: table slots at the load factor, the store
// slot and the per-state cluster / label word.
double bytes_per_state(const gpx_model *m, const BatchConfig &cfg) {
    const double load_factor = cfg.load_factor;
    const double sb = kSlotBytes[slot_kind(m, cfg.narrow_slots)];
    return sb / load_factor + sb + 4.0;
}

// Admission estimate: the state budget with a margin for the last level's
// overshoot, bounded by the product of the local state counts.
uint64_t estimate_capacity(const gpx_model *m, const gpx_batch_job &j) {
    double prod = 1;
    for (uint32_t ns : m->dec.nstates) prod *= ns;
    double est = j.max_states ? (double)j.max_states * 6.0 : 4.0e6; // a BFS level can overshoot the budget
    if (prod < est) est = prod * 1.05 + 64;
    if (est < 1024) est = 1024;
    return (uint64_t)est;
}

// Record init -> while (instances left) { batch_kernel; batch_relaunch_kernel } -> set hashes.
cudaError_t capture_batch(cudaStream_t st, BParams BP, int blocks, int threads, size_t smem, cudaEvent_t ev0,
                          cudaEvent_t ev1, uint32_t count, const BInst *d_inst, const uint32_t *d_words,
                          unsigned long long *d_hash, cudaGraph_t *out) {
    cudaStream_t sb = nullptr;
    bool body_open = false;
    cudaError_t e = cudaStreamCreateWithFlags(&sb, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    auto record = [&]() -> cudaError_t {
        cudaError_t r;
#define GPX_BCAP(call)                                                                                        \
    do {                                                                                                      \
        if ((r = (call)) != cudaSuccess) return r;                                                            \
    } while (0)
        GPX_BCAP(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        GPX_BCAP(cudaEventRecordWithFlags(ev0, st, cudaEventRecordExternal));
        batch_init_kernel<<<(count + 127) / 128, 128, 0, st>>>(BP, 1);
        GPX_BCAP(cudaGetLastError());
        cudaStreamCaptureStatus cs;
        cudaGraph_t g = nullptr;
        const cudaGraphNode_t *deps = nullptr;
        const cudaGraphEdgeData *edges = nullptr;
        size_t ndeps = 0;
        GPX_BCAP(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &edges, &ndeps));
        cudaGraphConditionalHandle loop;
        GPX_BCAP(cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams np = {cudaGraphNodeTypeConditional}; // the rest zero-initialised
        np.conditional.handle = loop;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        GPX_BCAP(cudaGraphAddNode(&node, g, deps, edges, ndeps, &np));
        GPX_BCAP(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
        GPX_BCAP(cudaStreamBeginCaptureToGraph(sb, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                               cudaStreamCaptureModeThreadLocal));
        body_open = true;
        void *args[] = {&BP};
        GPX_BCAP(cudaLaunchKernel((const void *)batch_kernel, dim3(blocks), dim3(threads), args, smem, sb));
        batch_relaunch_kernel<<<1, 1, 0, sb>>>(BP.g, count, loop);
        GPX_BCAP(cudaGetLastError());
        cudaGraph_t body = nullptr; // owned by the conditional node
        body_open = false;
        GPX_BCAP(cudaStreamEndCapture(sb, &body));
        GPX_BCAP(cudaEventRecordWithFlags(ev1, st, cudaEventRecordExternal));
        batch_hash_kernel<<<std::min<uint32_t>(count, 4096), 256, 0, st>>>(d_inst, count, d_words, d_hash);
        GPX_BCAP(cudaGetLastError());
#undef GPX_BCAP
        return cudaStreamEndCapture(st, out);
    };
    e = record();
    if (e != cudaSuccess) {
        cudaGraph_t t = nullptr;
        if (body_open) cudaStreamEndCapture(sb, &t);
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
            t = nullptr;
            cudaStreamEndCapture(st, &t);
            if (t) cudaGraphDestroy(t);
        }
        cudaGetLastError();
    }
    cudaStreamDestroy(sb);
    return e;
}

// One admission round: a graph with the batch_kernel launch loop over `idx`
// instances with the given capacities.
int run_launch(int device, const cudaDeviceProp &prop, const BatchConfig &cfg, uint64_t seed,
               const gpx_model *const *models, const gpx_batch_job *jobs, const std::vector<uint32_t> &idx,
               const std::vector<uint64_t> &cap, const gpx_por_model *d_por, std::vector<Outcome> *out,
               float *device_ms, uint32_t *launches) {
    int rc = GPX_OK;
    const uint32_t count = (uint32_t)idx.size();
    std::vector<BInst> h(count);
    std::vector<uint32_t> words_per(count);
    size_t table_bytes = 0, store_bytes = 0, sel_bytes = 0, model_words = 0;
    std::vector<size_t> toff(count), soff(count), seloff(count), moff(count);
    std::vector<size_t> ooff(count);
    size_t over_bytes = 0;
    for (uint32_t k = 0; k < count; k++) {
        const gpx_model *m = models[idx[k]];
        const uint32_t kind = slot_kind(m, cfg.narrow_slots), sb = kSlotBytes[kind], per_bucket = 32 / sb;
        uint64_t slots = (uint64_t)((double)cap[k] / cfg.load_factor) + 4;
        uint64_t nb = (slots + per_bucket - 1) / per_bucket;
        nb = (nb + 1) & ~1ull; // even: buckets are probed in pairs
        toff[k] = table_bytes;
        table_bytes += nb * 32;
        soff[k] = store_bytes;
        store_bytes += (cap[k] * sb + 255) & ~(size_t)255;
        ooff[k] = over_bytes;
        over_bytes += kInstOverflow * sb;
        seloff[k] = sel_bytes;
        const bool aux = jobs[idx[k]].por ? jobs[idx[k]].cycle_proviso != 0 : cfg.prune_commuting;
        if (aux) sel_bytes += (cap[k] * 4 + 255) & ~(size_t)255;
        moff[k] = model_words;
        model_words += (m->dec.words.size() + 63) & ~(size_t)63;
        memset(&h[k], 0, sizeof(BInst));
        h[k].nbuckets = nb;
        h[k].store_cap = cap[k];
        h[k].max_states = jobs[idx[k]].max_states;
        int prop_k = jobs[idx[k]].property;
        if (prop_k == GPX_PROP_SAFETY && m->gpf.liveness == 1) prop_k = GPX_PROP_LIVENESS;
        h[k].property = (uint32_t)prop_k;
        h[k].mode = jobs[idx[k]].por ? (jobs[idx[k]].cycle_proviso ? MODE_PROVISO : MODE_POR) : MODE_PLAIN;
        h[k].por_kind = jobs[idx[k]].por == 3 ? POR_AMPLE : (jobs[idx[k]].por == 4 ? POR_STUBBORN : POR_CAMPLE);
        h[k].kind = kind;
        h[k].ctrl.store_count = 1;
        h[k].ctrl.nlevels = 1;
        h[k].ctrl.hi = 1;
        h[k].lvl[0].lo = 0;
        h[k].lvl[0].hi = 1;
        h[k].lvl[0].phase = h[k].mode == MODE_PROVISO ? PH_DECIDE : PH_EXPAND;
        words_per[k] = m->dec.key_words;
    }
    unsigned char *d_table = nullptr, *d_store = nullptr, *d_sel = nullptr, *d_over = nullptr;
    uint32_t *d_models = nullptr, *d_words = nullptr;
    unsigned long long *d_levels = nullptr, *d_hash = nullptr;
    BInst *d_inst = nullptr;
    BGlobal *d_g = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaStream_t st = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<uint32_t> hm(model_words, 0);
    BParams BP;
    size_t smem = 0;
    int blocks = 0;
    std::vector<unsigned long long> hh(count, 0);
    std::vector<uint64_t> hl;
    for (uint32_t k = 0; k < count; k++) {
        const auto &w = models[idx[k]]->dec.words;
        std::copy(w.begin(), w.end(), hm.begin() + moff[k]);
    }
    BCUDA(cudaMalloc(&d_table, std::max<size_t>(table_bytes, 256)));
    BCUDA(cudaMalloc(&d_store, std::max<size_t>(store_bytes, 256)));
    BCUDA(cudaMalloc(&d_sel, std::max<size_t>(sel_bytes, 256)));
    BCUDA(cudaMalloc(&d_over, std::max<size_t>(over_bytes, 256)));
    BCUDA(cudaMalloc(&d_models, std::max<size_t>(model_words * 4, 256)));
    BCUDA(cudaMalloc(&d_words, count * 4));
    BCUDA(cudaMalloc(&d_levels, (size_t)count * kBatchLevels * 8));
    BCUDA(cudaMalloc(&d_hash, count * 8));
    BCUDA(cudaMalloc(&d_inst, count * sizeof(BInst)));
    BCUDA(cudaMalloc(&d_g, sizeof(BGlobal)));
    for (uint32_t k = 0; k < count; k++) {
        h[k].por_model = (jobs[idx[k]].por == 2) ? d_por : nullptr;
        h[k].table = d_table + toff[k];
        h[k].store = d_store + soff[k];
        const bool aux = h[k].mode == MODE_PROVISO || (h[k].mode == MODE_PLAIN && cfg.prune_commuting);
        h[k].aux = aux ? (uint32_t *)(d_sel + seloff[k]) : nullptr;
        h[k].model = d_models + moff[k];
        h[k].levels = d_levels + (size_t)k * kBatchLevels;
        h[k].overflow = d_over + ooff[k];
        h[k].overflow_cap = kInstOverflow;
    }
    BCUDA(cudaMemset(d_table, 0, std::max<size_t>(table_bytes, 256)));
    BCUDA(cudaMemset(d_hash, 0, count * 8));
    BCUDA(cudaMemset(d_g, 0, sizeof(BGlobal)));
    BCUDA(cudaMemcpy(d_models, hm.data(), model_words * 4, cudaMemcpyHostToDevice));
    BCUDA(cudaMemcpy(d_words, words_per.data(), count * 4, cudaMemcpyHostToDevice));
    BCUDA(cudaMemcpy(d_inst, h.data(), count * sizeof(BInst), cudaMemcpyHostToDevice));
    memset(&BP, 0, sizeof BP);
    BP.inst = d_inst;
    BP.g = d_g;
    BP.count = count;
    BP.claim = (uint32_t)cfg.claim;
    BP.max_claims = (uint32_t)std::max(0, cfg.kernel_iters);
    BP.seed = seed;
    BP.timeout_ns = 20ull * 1000 * 1000 * 1000;
    // only with a full grid: every SM, the reserved ones included, then hosts blocks
    BP.latency_sms =
        cfg.blocks > 0 ? 0u : (uint32_t)std::max(0, std::min(cfg.latency_sms, prop.multiProcessorCount / 2));
    smem = (size_t)(cfg.threads / 32) * sizeof(WarpScratch<K128, MODE_PROVISO>);
    BCUDA(cudaFuncSetAttribute((const void *)batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    {
        int per_sm = 0;
        BCUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)batch_kernel, cfg.threads, smem));
        blocks = cfg.blocks > 0 ? cfg.blocks : std::max(1, per_sm) * prop.multiProcessorCount;
    }
    BP.total_warps = (uint32_t)(blocks * (cfg.threads / 32));
    BCUDA(cudaEventCreate(&ev0));
    BCUDA(cudaEventCreate(&ev1));
    BCUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    // One graph: init, a device-side while loop over batch_kernel launches
    // (batch_relaunch_kernel decides whether another follows), set hashes.
    {
        cudaError_t ce = capture_batch(st, BP, blocks, cfg.threads, smem, ev0, ev1, count, d_inst, d_words, d_hash,
                                       &graph);
        if (ce == cudaSuccess) ce = cudaGraphInstantiate(&exec, graph, 0);
        if (ce != cudaSuccess) {
            fprintf(stderr, "gpx batch: building the launch graph failed: %s\n", cudaGetErrorString(ce));
            cudaGetLastError();
            rc = GPX_ERR_CUDA;
            goto done;
        }
    }
    BCUDA(cudaGraphLaunch(exec, st));
    BCUDA(cudaStreamSynchronize(st));
    {
        float ms = 0;
        cudaEventElapsedTime(&ms, ev0, ev1);
        *device_ms += ms;
        BGlobal g;
        BCUDA(cudaMemcpy(&g, d_g, sizeof g, cudaMemcpyDeviceToHost));
        *launches += (uint32_t)g.launches;
        if (g.error) rc = (int)g.error;
    }
    BCUDA(cudaMemcpy(h.data(), d_inst, count * sizeof(BInst), cudaMemcpyDeviceToHost));
    BCUDA(cudaMemcpy(hh.data(), d_hash, count * 8, cudaMemcpyDeviceToHost));
    hl.resize((size_t)count * kBatchLevels);
    BCUDA(cudaMemcpy(hl.data(), d_levels, hl.size() * 8, cudaMemcpyDeviceToHost));
    {
        BGlobal g;
        BCUDA(cudaMemcpy(&g, d_g, sizeof g, cudaMemcpyDeviceToHost));
        out->resize(count);
        for (uint32_t k = 0; k < count; k++) {
            Outcome &o = (*out)[k];
            const Ctrl &c = h[k].ctrl;
            o.status = c.error ? (int)c.error : (c.done ? GPX_OK : (rc ? rc : GPX_ERR_TIMEOUT));
            o.stopped = c.error ? GPX_STOP_ERROR : (int)c.stop;
            o.verdict = (c.done && c.stop == GPX_STOP_VIOLATION) ? (int)h[k].property : GPX_PROP_NONE;
            o.states = std::min<unsigned long long>(c.store_count, h[k].store_cap);
            o.nlevels = c.nlevels;
            o.set_hash = hh[k];
            o.capacity = cap[k];
            o.completion_ms = h[k].finish_ns > g.start_ns ? (h[k].finish_ns - g.start_ns) * 1e-6 : 0.0;
            o.levels.assign(hl.begin() + (size_t)k * kBatchLevels,
                            hl.begin() + (size_t)k * kBatchLevels + std::min<uint32_t>(c.nlevels, kBatchLevels));
        }
    }
done:
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (st) cudaStreamDestroy(st);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    cudaFree(d_table);
    cudaFree(d_store);
    cudaFree(d_sel);
    cudaFree(d_over);
    cudaFree(d_models);
    cudaFree(d_words);
    cudaFree(d_levels);
    cudaFree(d_hash);
    cudaFree(d_inst);
    cudaFree(d_g);
    return rc;
}

double percentile(std::vector<double> v, double q) {
    if (v.empty()) return 0;
    std::sort(v.begin(), v.end());
    size_t i = (size_t)std::min<double>(v.size() - 1, std::max(0.0, q * (v.size() - 1) + 0.5));
    return v[i];
}

} // namespace

extern "C" {

void gpx_batch_options_init(gpx_batch_options *o) {
    memset(o, 0, sizeof *o);
    o->struct_size = sizeof *o;
    o->seed = 0x243F6A8885A308D3ull;
    o->latency_sms = -1;
    o->prune_commuting = 1;
}

void gpx_batch_job_init(gpx_batch_job *j) {
    memset(j, 0, sizeof *j);
    j->struct_size = sizeof *j;
}

int gpx_batch_explore(const gpx_model *const *models, const gpx_batch_job *jobs, uint32_t count,
                      const gpx_batch_options *opts, gpx_batch_item *items, uint64_t *level_counts,
                      uint32_t level_capacity, gpx_batch_stats *stats) {
    if (!models || !jobs || !items || !opts || !count || opts->struct_size != sizeof(gpx_batch_options))
        return GPX_ERR_INVALID;
    if (opts->threads < 0 || opts->threads % 32 || opts->threads > 256 || opts->load_factor > 0.95)
        return GPX_ERR_INVALID; // refused before a GPU is looked for
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GPX_ERR_NO_GPU;
    if (opts->device < 0 || opts->device >= ndev) return GPX_ERR_INVALID;
    if (cudaSetDevice(opts->device) != cudaSuccess) return GPX_ERR_CUDA;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, opts->device) != cudaSuccess) return GPX_ERR_CUDA;
    BatchConfig cfg;
    cfg.blocks = opts->blocks;
    cfg.threads = opts->threads > 0 ? opts->threads : 256;
    cfg.claim = opts->claim > 0 ? opts->claim : 8;
    cfg.narrow_slots = opts->narrow_slots != 0;
    cfg.kernel_iters = opts->kernel_iters;
    cfg.load_factor = opts->load_factor > 0 ? opts->load_factor : 0.5;
    // automatic: about a tenth of the SMs (16 of 152 measured best on config 5, with 8
    // and 24 worse); 0 switches the reservation off
    cfg.latency_sms = opts->latency_sms >= 0 ? opts->latency_sms : prop.multiProcessorCount / 10 + 1;
    cfg.prune_commuting = opts->prune_commuting != 0;
    const int max_adm = opts->max_admissions > 0 ? opts->max_admissions : 3;
    gpx_batch_stats st;
    memset(&st, 0, sizeof st);

    std::vector<uint32_t> todo;
    std::vector<uint64_t> cap(count, 0);
    for (uint32_t i = 0; i < count; i++) {
        memset(&items[i], 0, sizeof items[i]);
        if (!models[i] || jobs[i].struct_size != sizeof(gpx_batch_job) || jobs[i].por < 0 || jobs[i].por > 4)
            return GPX_ERR_INVALID;
        // an instance too wide for 128-bit slots, or with a liveness property (the
        // accepting-cycle check runs through gpx_explorer_run only)
        if (models[i]->dec.state_bits > (uint32_t)kMaxStateBits ||
            (jobs[i].property == GPX_PROP_SAFETY && models[i]->gpf.liveness == 1) ||
            jobs[i].property == GPX_PROP_LIVENESS) {
            items[i].status = GPX_ERR_UNSUPPORTED;
            items[i].stopped = GPX_STOP_ERROR;
            continue;
        }
        cap[i] = jobs[i].capacity ? jobs[i].capacity : estimate_capacity(models[i], jobs[i]);
        todo.push_back(i);
    }
    // Admission: the estimates of one launch must fit in device memory (table at the
    // load factor + store + cluster array per state); scale them down together if
    // not -- instances that then overflow are re-admitted with more room.
    {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return GPX_ERR_CUDA;
        double want = 0;
        for (uint32_t i : todo) want += (double)cap[i] * bytes_per_state(models[i], cfg);
        const double room = 0.7 * (double)free_b;
        if (want > room)
            for (uint32_t i : todo) cap[i] = std::max<uint64_t>(1024, (uint64_t)((double)cap[i] * room / want));
    }
    gpx_por_model *d_por = nullptr;
    if (opts->por_model) {
        if (cudaMalloc(&d_por, sizeof(gpx_por_model)) != cudaSuccess) return GPX_ERR_NOMEM;
        cudaMemcpy(d_por, opts->por_model, sizeof(gpx_por_model), cudaMemcpyHostToDevice);
    }
    // the request rate of random hash probes bounds these kernels: fetch one sector per L2 miss
    size_t saved_fetch = 0;
    bool restore = cudaDeviceGetLimit(&saved_fetch, cudaLimitMaxL2FetchGranularity) == cudaSuccess &&
                   cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, 32) == cudaSuccess;

    if (opts->autotune && todo.size() > 1) {
        // tune on a sample of at most 64 instances, spread over the batch with a
        // stride coprime to its size: an even stride over a batch whose job kinds
        // alternate with the index sampled one kind only
        auto t0 = std::chrono::steady_clock::now();
        std::vector<uint32_t> sample;
        const size_t nt = todo.size(), want = std::min<size_t>(nt, 64);
        size_t stride = std::max<size_t>(1, nt / want) | 1;
        while (std::gcd(stride, nt) != 1) stride += 2;
        for (size_t k = 0; k < want; k++) sample.push_back(todo[(k * stride) % nt]);
        std::sort(sample.begin(), sample.end());
        std::vector<uint64_t> scap;
        for (uint32_t i : sample) scap.push_back(cap[i]);
        double best = 1e30;
        BatchConfig bestc = cfg;
        // (claims of 4 states suit batches of latency-bound rings, 16 the mixed
        // config-5 batch: 0.79 / 385 ms against 0.83 / 415 ms with 8)
        for (int threads : {128, 256})
            for (int claim : {4, 8, 16, 32, 64, 256})
                for (double lf : {0.25, 0.5}) {
                    BatchConfig c = cfg;
                    c.threads = threads;
                    c.claim = claim;
                    c.load_factor = lf;
                    std::vector<Outcome> o;
                    float ms = 0;
                    uint32_t l = 0;
                    if (run_launch(opts->device, prop, c, opts->seed, models, jobs, sample, scap, d_por, &o, &ms,
                                   &l) ==
                            GPX_OK &&
                        ms < best) {
                        best = ms;
                        bestc = c;
                    }
                }
        // then the claims per warp per launch (0: one launch until every instance is
        // done; otherwise warps leave after that many claims and the device-side
        // loop relaunches, which redistributes them over the SMs)
        for (int iters : {0, 64, 512}) {
            if (iters == bestc.kernel_iters) continue;
            BatchConfig c = bestc;
            c.kernel_iters = iters;
            std::vector<Outcome> o;
            float ms = 0;
            uint32_t l = 0;
            if (run_launch(opts->device, prop, c, opts->seed, models, jobs, sample, scap, d_por, &o, &ms, &l) ==
                    GPX_OK &&
                ms < best) {
                best = ms;
                bestc = c;
            }
        }
        {   // then the slot policy: narrow slots save memory, 128-bit slots are often faster
            BatchConfig c = bestc;
            c.narrow_slots = !bestc.narrow_slots;
            std::vector<Outcome> o;
            float ms = 0;
            uint32_t l = 0;
            if (run_launch(opts->device, prop, c, opts->seed, models, jobs, sample, scap, d_por, &o, &ms, &l) ==
                    GPX_OK &&
                ms < best) {
                best = ms;
                bestc = c;
            }
        }
        // Last, the claim size on the whole batch (at most 1,024 instances), at
        // the sample's choice and two and four times it: a batch's makespan is
        // set by its deepest instances, which a sample rarely holds (config 5:
        // 608 ms with 16-state claims against 640 with the sample's 8).  A run in
        // which an instance outgrew its partition still times the launch.
        if (sample.size() < todo.size() && todo.size() <= 1024) {
            double full_best = 1e30;
            BatchConfig full_c = bestc;
            std::vector<uint64_t> fcap; // admission capacities, in the order of todo
            for (uint32_t i : todo) fcap.push_back(cap[i]);
            for (int mul : {1, 2, 4}) {
                BatchConfig c = bestc;
                c.claim = bestc.claim * mul;
                if (c.claim > 256) break;
                std::vector<Outcome> o;
                float ms = 0;
                uint32_t l = 0;
                const int r = run_launch(opts->device, prop, c, opts->seed, models, jobs, todo, fcap, d_por, &o, &ms, &l);
                if ((r == GPX_OK || r == GPX_ERR_TABLE_FULL || r == GPX_ERR_STORE_FULL) && ms < full_best) {
                    full_best = ms;
                    full_c = c;
                }
            }
            bestc = full_c;
        }
        cfg = bestc;
        st.tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }

    int rc = GPX_OK;
    std::vector<double> completion;
    for (int adm = 1; adm <= max_adm && !todo.empty(); adm++) {
        std::vector<uint64_t> c2;
        {
            size_t free_b = 0, total_b = 0;
            cudaMemGetInfo(&free_b, &total_b);
            double want = 0;
            for (uint32_t i : todo) want += (double)cap[i] * bytes_per_state(models[i], cfg);
            const double room = 0.7 * (double)free_b;
            double scale = want > room ? room / want : 1.0;
            for (uint32_t i : todo) c2.push_back(std::max<uint64_t>(1024, (uint64_t)((double)cap[i] * scale)));
        }
        std::vector<Outcome> out;
        float ms = 0;
        rc = run_launch(opts->device, prop, cfg, opts->seed, models, jobs, todo, c2, d_por, &out, &ms, &st.launches);
        st.device_ms += ms;
        if (rc != GPX_OK && out.empty()) break;
        std::vector<uint32_t> again;
        for (size_t k = 0; k < todo.size(); k++) {
            uint32_t i = todo[k];
            const Outcome &o = out[k];
            gpx_batch_item &it = items[i];
            it.admissions = (uint32_t)adm;
            it.status = o.status;
            it.stopped = o.stopped;
            it.verdict = o.verdict;
            it.states = o.states;
            it.nlevels = o.nlevels;
            it.set_hash = o.set_hash;
            it.capacity = o.capacity;
            it.completion_ms = o.completion_ms;
            it.slot_bytes = kSlotBytes[slot_kind(models[i], cfg.narrow_slots)];
            if (adm == 1 && o.status == GPX_OK) completion.push_back(o.completion_ms);
            if (level_counts && level_capacity)
                for (uint32_t l = 0; l < std::min<uint32_t>(level_capacity, (uint32_t)o.levels.size()); l++)
                    level_counts[(size_t)i * level_capacity + l] = o.levels[l];
            if ((o.status == GPX_ERR_TABLE_FULL || o.status == GPX_ERR_STORE_FULL) && adm < max_adm) {
                cap[i] *= 4; // re-admit with a bigger partition
                again.push_back(i);
            }
        }
        todo.swap(again);
        if (rc != GPX_OK && rc != GPX_ERR_TABLE_FULL && rc != GPX_ERR_STORE_FULL) break;
        rc = GPX_OK;
    }
    if (restore) cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, saved_fetch);
    if (d_por) cudaFree(d_por);
    for (uint32_t i = 0; i < count; i++) st.states += items[i].states;
    st.p50_ms = percentile(completion, 0.50);
    st.p99_ms = percentile(completion, 0.99);
    st.claim = cfg.claim;
    st.threads = cfg.threads;
    st.blocks = cfg.blocks;
    st.load_factor = cfg.load_factor;
    st.kernel_iters = cfg.kernel_iters;
    st.narrow_slots = cfg.narrow_slots ? 1 : 0;
    for (uint32_t i = 0; i < count; i++)
        if (items[i].slot_bytes) st.instances_by_slot[items[i].slot_bytes == 4 ? 0 : (items[i].slot_bytes == 8 ? 1 : 2)]++;
    if (stats) *stats = st;
    return rc;
}

} // extern "C"
