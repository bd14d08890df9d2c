// gpx_device.cuh -- device building blocks shared by the exploration kernels:
// slot/key traits, the bucketised hash table, per-warp scratch and the per-warp
// expansion engine (Explorer).  Included by gpx_explore.cu (single network) and
// gpx_batch.cu (many networks in one launch).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "gpx.h"
#include "gpx_model.h"

namespace gpx {

// ------------------------------------------------------------------ constants

constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr int kPairMax = 256;   // (state, process) pairs staged per warp batch
constexpr int kPairMaxPor = 160; // ... with POR: its per-pair arrays then fit 4 blocks per SM
static_assert(kPairMax <= 256 && kPairMaxPor <= 256, "successor owners are stored as 8-bit pair indices");
constexpr int kMaxProbe = 32;   // buckets probed before reporting the table full
constexpr uint32_t kMaxLevels = 1u << 20;
// cluster definitions of the POR modes: static clusters (cample), single-process
// clusters only (ample), state-dependent necessary-enabling clusters (stubborn)
enum PorKind : uint32_t { POR_CAMPLE = 0, POR_AMPLE = 1, POR_STUBBORN = 2 };
constexpr unsigned long long kMaxLaunches = 2ull * kMaxLevels; // exploration launches per run

enum Mode : int { MODE_PLAIN = 0, MODE_POR = 1, MODE_PROVISO = 2 };
// A level's phases: the cycle proviso's lookup pass (DECIDE), the expansion
// with inserts (EXPAND), and -- only when some insert found its whole probe
// sequence full -- the placement of those keys with eviction (PLACE).
enum Phase : uint32_t { PH_EXPAND = 0, PH_DECIDE = 1, PH_PLACE = 2 };
constexpr int kEvictDepth = 4; // displacements one placement may chain

// Control block shared by all blocks of the persistent kernel.
// Run control block.  Fields that many warps touch during a level sit on
// separate 128-byte lines: the level parameters (written only by the thread
// that closes a phase), the claim cursor, the store append counter, the two
// barrier words and the statistics, so polling and atomics on one do not queue
// behind the others in the same L2 slice.
struct alignas(128) Ctrl {
    unsigned long long lo, hi;      // the level being expanded: store indices [lo, hi)
    unsigned int claim;             // states per claim
    unsigned int level;             // BFS depth of [lo, hi)
    unsigned int nlevels;           // recorded level counts
    unsigned int done;              // exploration finished
    unsigned int pause;             // launch budget (-k) reached: kernel returns, host relaunches
    unsigned int violation;         // property violated during this level
    unsigned int error;             // gpx_status
    unsigned int stop;              // gpx_stop
    unsigned int phase;             // Phase
    unsigned int launch_levels;     // levels closed in this launch
    unsigned int timeout_at;        // where a bounded wait gave up (diagnostics)
    unsigned int tag;               // generation of this run's keys (tagged 128-bit slots; else 0)
    unsigned long long overflow_count; // keys whose probe sequence was full during this level
    unsigned long long evictions;      // keys displaced to make room
    unsigned long long launches;       // exploration launches of a graph-driven run
    unsigned long long overflowed;     // keys that went through a placement phase (whole run)
    unsigned long long place_ns;       // device time of the placement phases (whole run)
    unsigned long long place_t0;       // start of the current placement phase
    unsigned int place_blocks;         // blocks of place_kernel that have finished
    alignas(128) unsigned long long cursor;      // dynamic claims: offset beyond the static first claims
    alignas(128) unsigned long long store_count; // states appended to the store
    alignas(128) unsigned int bar_count;         // grid barrier arrivals
    alignas(128) unsigned long long bar_word;    // grid barrier: generation and the next phase (polled)
    alignas(128) unsigned long long lookups; // statistics (one line)
    unsigned long long probes, expanded, inserts, inserts_lookups, pruned;
};

struct Params {
    void *table;
    unsigned long long nbuckets;
    void *store;
    unsigned long long store_cap;
    const uint32_t *model; // device layout (gpx_model.h)
    uint32_t model_words;
    uint32_t model_in_smem;
    uint32_t *sel;         // per-frontier-state cluster (cycle proviso)
    unsigned long long *levels;
    Ctrl *ctrl;
    unsigned long long seed;
    unsigned long long max_states;
    unsigned long long timeout_ns;
    uint32_t property;
    uint32_t levels_per_launch;
    uint32_t total_warps;
    uint32_t batch_states;  // states in a warp's full batch (pairs per batch / processes, at most 32)
    uint32_t por_kind;      // POR_CAMPLE, POR_AMPLE or POR_STUBBORN
    // keys whose probe sequence was full, placed with eviction in a phase of their own
    void *overflow;
    unsigned long long overflow_cap;
    // 128-bit claim entries {epoch, overflow index} deduplicating the overflow list
    // ([0] holds the epoch counter, which survives runs); null: placement by one warp
    unsigned long long *claim;
    unsigned long long claim_cap; // entries, a power of two
    // learned cluster proposal (por == 2) and candidate logging (decide pass)
    const gpx_por_model *por_model;
    uint32_t learned;
    uint32_t log_every;
    gpx_por_log_row *log;
    unsigned long long *log_count;
    unsigned long long log_cap;
    // tagged slots: the generation counter the init kernel steps (null: untagged)
    unsigned long long *gen;
    // plain mode: per store position, the participants of the move that first
    // inserted the state (0: none); null disables commuting-move pruning
    uint32_t *label;
};

// ------------------------------------------------------------- device helpers

static __device__ __forceinline__ uint64_t mix64(uint64_t z) { // SplitMix64 finaliser (Steele, Lea, Flood 2014)
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static __device__ __forceinline__ uint64_t globaltimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

static __device__ __forceinline__ void set_error(Ctrl *c, unsigned int code) { atomicCAS(&c->error, 0u, code); }

static __device__ __forceinline__ void prefetch_l2(const void *p) {
    asm volatile("prefetch.global.L2 [%0];" : : "l"(p));
}

// One 32-byte bucket in one load.  Each vector element is read single-copy
// atomically, so a slot is never seen half-written: 32-bit elements for
// 32-bit slots, 64-bit elements for 64-bit slots and the halves of 128-bit ones.
static __device__ __forceinline__ void ld256_cg(const void *p, uint32_t (&w)[8]) {
    asm volatile("ld.global.cg.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]), "=r"(w[6]), "=r"(w[7])
                 : "l"(p));
}

static __device__ __forceinline__ void ld256_cg(const void *p, unsigned long long (&d)[4]) {
    asm volatile("ld.global.cg.v4.u64 {%0,%1,%2,%3}, [%4];"
                 : "=l"(d[0]), "=l"(d[1]), "=l"(d[2]), "=l"(d[3])
                 : "l"(p));
}

static __device__ __forceinline__ uint64_t lmask(uint32_t w) { return (w >= 64) ? ~0ull : ((1ull << w) - 1ull); }

// Keys are stored in slot form: the packed state vector plus an occupancy
// marker in the top bit of each 32/64-bit half, so an all-zero slot is empty
// and the all-zero state vector is a valid key.
struct K32 { uint32_t v; };
struct K64 { unsigned long long v; };
struct __align__(16) K128 { unsigned long long lo, hi; };

template <class K> struct KT;

template <> struct KT<K32> {
    static constexpr int kSlots = 8; // 32-byte bucket
    __device__ static K32 initial(uint32_t) { return {0x80000000u}; }
    __device__ static uint32_t tag_of(const K32 &) { return 0; }
    __device__ static bool eq(const K32 &a, const K32 &b) { return a.v == b.v; }
    __device__ static bool empty(const K32 &a, uint32_t) { return a.v == 0; }
    __device__ static bool torn(const K32 &, uint32_t) { return false; }
    __device__ static uint32_t get(const K32 &k, uint32_t f, uint32_t w) { return (k.v >> f) & (uint32_t)lmask(w); }
    __device__ static void set(K32 &k, uint32_t f, uint32_t w, uint32_t x) {
        uint32_t m = (uint32_t)lmask(w) << f;
        k.v = (k.v & ~m) | ((x << f) & m);
    }
    __device__ static uint64_t hash(const K32 &k, uint64_t seed) { return mix64((uint64_t)k.v ^ seed); }
    __device__ static K32 cas(K32 *p, K32 cmp, K32 val) { return {atomicCAS(&p->v, cmp.v, val.v)}; }
    __device__ static void bucket(const K32 *b, K32 (&s)[kSlots]) {
        uint32_t w[8];
        ld256_cg(b, w);
#pragma unroll
        for (int j = 0; j < 8; j++) s[j].v = w[j];
    }
    __device__ static K32 load(const K32 *p) { return {__ldcg(&p->v)}; }
    __device__ static void words(const K32 &k, uint32_t (&w)[4]) {
        w[0] = k.v & 0x7FFFFFFFu;
        w[1] = w[2] = w[3] = 0;
    }
};

template <> struct KT<K64> {
    static constexpr int kSlots = 4; // 32-byte bucket
    __device__ static K64 initial(uint32_t) { return {0x8000000000000000ull}; }
    __device__ static uint32_t tag_of(const K64 &) { return 0; }
    __device__ static bool eq(const K64 &a, const K64 &b) { return a.v == b.v; }
    __device__ static bool empty(const K64 &a, uint32_t) { return a.v == 0; }
    __device__ static bool torn(const K64 &, uint32_t) { return false; }
    __device__ static uint32_t get(const K64 &k, uint32_t f, uint32_t w) { return (uint32_t)((k.v >> f) & lmask(w)); }
    __device__ static void set(K64 &k, uint32_t f, uint32_t w, uint32_t x) {
        unsigned long long m = lmask(w) << f;
        k.v = (k.v & ~m) | (((unsigned long long)x << f) & m);
    }
    __device__ static uint64_t hash(const K64 &k, uint64_t seed) { return mix64(k.v ^ seed); }
    __device__ static K64 cas(K64 *p, K64 cmp, K64 val) { return {atomicCAS(&p->v, cmp.v, val.v)}; }
    __device__ static void bucket(const K64 *b, K64 (&s)[kSlots]) {
        unsigned long long d[4];
        ld256_cg(b, d);
#pragma unroll
        for (int j = 0; j < 4; j++) s[j].v = d[j];
    }
    __device__ static K64 load(const K64 *p) { return {__ldcg(&p->v)}; }
    __device__ static void words(const K64 &k, uint32_t (&w)[4]) {
        unsigned long long v = k.v & 0x7FFFFFFFFFFFFFFFull;
        w[0] = (uint32_t)v;
        w[1] = (uint32_t)(v >> 32);
        w[2] = w[3] = 0;
    }
};

// Shared by the two 128-bit slot forms: the state vector is split into a low
// part of S bits (in the low 64-bit half) and the rest (in the high half).
template <uint32_t S> struct Split128 {
    // Without branches (the lanes of a warp read fields of different halves):
    // the state vector as one 2S-bit value x1:x0, then a funnel shift.
    __device__ static uint32_t get(unsigned long long lo, unsigned long long hi, uint32_t f, uint32_t w) {
        constexpr unsigned long long m = (1ull << S) - 1ull;
        const unsigned long long h = hi & m;
        const unsigned long long x0 = (lo & m) | (h << S), x1 = h >> (64 - S);
        const unsigned long long v = f >= 64 ? (x1 >> (f - 64)) : ((x0 >> f) | ((x1 << 1) << (63 - f)));
        return (uint32_t)(v & lmask(w));
    }
    __device__ static void set(unsigned long long &lo, unsigned long long &hi, uint32_t f, uint32_t w, uint32_t x) {
        if (f + w <= S) {
            unsigned long long m = lmask(w) << f;
            lo = (lo & ~m) | (((unsigned long long)x << f) & m);
        } else if (f >= S) {
            unsigned long long m = lmask(w) << (f - S);
            hi = (hi & ~m) | (((unsigned long long)x << (f - S)) & m);
        } else {
            uint32_t nlo = S - f;
            unsigned long long ml = lmask(nlo) << f, mh = lmask(w - nlo);
            lo = (lo & ~ml) | (((unsigned long long)x << f) & ml);
            hi = (hi & ~mh) | (((unsigned long long)x >> nlo) & mh);
        }
    }
    // the state vector as 32-bit words (lo and hi hold state bits only)
    __device__ static void words(unsigned long long lo, unsigned long long hi, uint32_t (&w)[4]) {
        w[0] = (uint32_t)lo;
        w[1] = (uint32_t)(lo >> 32) | (uint32_t)(hi << (S - 32));
        w[2] = (uint32_t)(hi >> (64 - S));
        w[3] = (uint32_t)(hi >> (96 - S));
    }
};

static __device__ __forceinline__ void cas128(void *p, unsigned long long clo, unsigned long long chi,
                                              unsigned long long vlo, unsigned long long vhi,
                                              unsigned long long &olo, unsigned long long &ohi) {
    asm volatile(
        "{\n\t.reg .b128 c, v, o;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 v, {%4, %5};\n\t"
        "atom.global.cas.b128 o, [%6], c, v;\n\t"
        "mov.b128 {%0, %1}, o;\n\t}"
        : "=l"(olo), "=l"(ohi)
        : "l"(clo), "l"(chi), "l"(vlo), "l"(vhi), "l"(p)
        : "memory");
}

static __device__ __forceinline__ void bucket128(const void *b, unsigned long long (&lo)[2],
                                                 unsigned long long (&hi)[2]) {
    unsigned long long d[4];
    ld256_cg(b, d);
    lo[0] = d[0];
    hi[0] = d[1];
    lo[1] = d[2];
    hi[1] = d[3];
}

// 128-bit slots hold 63 state bits in each 64-bit half (bit 63 of both halves
// is the occupancy marker).  Each half is read atomically, so a slot caught in
// the middle of its insertion shows exactly one zero half ("torn"); such a slot
// is re-read with an atomic before it is judged.
template <> struct KT<K128> {
    static constexpr int kSlots = 2; // 32-byte bucket
    static constexpr unsigned long long kOcc = 0x8000000000000000ull;
    using Sp = Split128<63>;
    __device__ static K128 initial(uint32_t) { return {kOcc, kOcc}; }
    __device__ static uint32_t tag_of(const K128 &) { return 0; }
    __device__ static bool eq(const K128 &a, const K128 &b) { return a.lo == b.lo && a.hi == b.hi; }
    __device__ static bool empty(const K128 &a, uint32_t) { return (a.lo | a.hi) == 0; }
    __device__ static bool torn(const K128 &a, uint32_t) { return (a.lo == 0) != (a.hi == 0); }
    __device__ static uint32_t get(const K128 &k, uint32_t f, uint32_t w) { return Sp::get(k.lo, k.hi, f, w); }
    __device__ static void set(K128 &k, uint32_t f, uint32_t w, uint32_t x) { Sp::set(k.lo, k.hi, f, w, x); }
    __device__ static uint64_t hash(const K128 &k, uint64_t seed) { return mix64(k.lo ^ mix64(k.hi ^ seed)); }
    __device__ static K128 cas(K128 *p, K128 cmp, K128 val) {
        K128 o;
        cas128(p, cmp.lo, cmp.hi, val.lo, val.hi, o.lo, o.hi);
        return o;
    }
    __device__ static void bucket(const K128 *b, K128 (&s)[kSlots]) {
        unsigned long long lo[2], hi[2];
        bucket128(b, lo, hi);
        s[0] = {lo[0], hi[0]};
        s[1] = {lo[1], hi[1]};
    }
    __device__ static K128 load(const K128 *p) { return {__ldcg(&p->lo), __ldcg(&p->hi)}; }
    __device__ static void words(const K128 &k, uint32_t (&w)[4]) { Sp::words(k.lo & ~kOcc, k.hi & ~kOcc, w); }
};

// 128-bit slots of a reusable table: 56 state bits in each 64-bit half and the
// run's generation (1..255) in the top byte of both halves.  A half carrying
// another generation -- or zero -- is free, so a new run needs no table clear:
// the table is zeroed on its first run and once every 255 runs.  During a run
// a slot still changes once, from free to a key of the run, by a full-slot CAS
// against the free contents it was read with.  Each half is read atomically, so
// a slot caught in the middle of its insertion shows exactly one half of the
// current generation ("torn") and is re-read with an atomic before it is judged.
// Keys carry the generation, and successors inherit it from their source state.
struct __align__(16) K128G { unsigned long long lo, hi; };

template <> struct KT<K128G> {
    static constexpr int kSlots = 2; // 32-byte bucket
    static constexpr uint32_t kStateBits = 56;
    static constexpr unsigned long long kMask = (1ull << kStateBits) - 1ull;
    using Sp = Split128<kStateBits>;
    __device__ static bool cur(unsigned long long h, uint32_t tag) { return (uint32_t)(h >> kStateBits) == tag; }
    __device__ static K128G initial(uint32_t tag) {
        const unsigned long long t = (unsigned long long)tag << kStateBits;
        return {t, t};
    }
    __device__ static uint32_t tag_of(const K128G &k) { return (uint32_t)(k.lo >> kStateBits); }
    __device__ static bool eq(const K128G &a, const K128G &b) { return a.lo == b.lo && a.hi == b.hi; }
    __device__ static bool empty(const K128G &a, uint32_t tag) { return !cur(a.lo, tag) && !cur(a.hi, tag); }
    __device__ static bool torn(const K128G &a, uint32_t tag) { return cur(a.lo, tag) != cur(a.hi, tag); }
    __device__ static uint32_t get(const K128G &k, uint32_t f, uint32_t w) { return Sp::get(k.lo, k.hi, f, w); }
    __device__ static void set(K128G &k, uint32_t f, uint32_t w, uint32_t x) { Sp::set(k.lo, k.hi, f, w, x); }
    __device__ static uint64_t hash(const K128G &k, uint64_t seed) {
        return mix64((k.lo & kMask) ^ mix64((k.hi & kMask) ^ seed));
    }
    __device__ static K128G cas(K128G *p, K128G cmp, K128G val) {
        K128G o;
        cas128(p, cmp.lo, cmp.hi, val.lo, val.hi, o.lo, o.hi);
        return o;
    }
    __device__ static void bucket(const K128G *b, K128G (&s)[kSlots]) {
        unsigned long long lo[2], hi[2];
        bucket128(b, lo, hi);
        s[0] = {lo[0], hi[0]};
        s[1] = {lo[1], hi[1]};
    }
    __device__ static K128G load(const K128G *p) { return {__ldcg(&p->lo), __ldcg(&p->hi)}; }
    __device__ static void words(const K128G &k, uint32_t (&w)[4]) { Sp::words(k.lo & kMask, k.hi & kMask, w); }
};

// Probe sequence of a key: 32-byte buckets visited in pairs -- a bucket, then
// its neighbour in the same 64-byte line -- for kMaxProbe/2 hash functions.
// The table holds an even number of buckets.
static __device__ __forceinline__ unsigned long long bucket_of(uint64_t h, int i, unsigned long long nb) {
    int j = i >> 1;
    uint64_t x = j ? mix64(h + (uint64_t)j * 0x9E3779B97F4A7C15ull) : h;
    unsigned long long b = __umul64hi(x, nb);
    return (i & 1) ? (b ^ 1ull) : b;
}

// Find-or-insert.  Returns 0 if the key was present, 1 if this call inserted
// it, 2 if every probed bucket was full.  Slots go from empty to a key exactly
// once during a level (keys move only in the placement phase, when no other
// thread inserts or looks up); every caller scans the same probe sequence and claims the first
// empty slot it sees with a full-key CAS against the contents it read, so two
// insertions of one key always meet in the same slot and exactly one wins.
template <class K>
__device__ __forceinline__ int find_or_insert(K *table, unsigned long long nb, const K &key, uint64_t h,
                                              unsigned int &probes) {
    constexpr int S = KT<K>::kSlots;
    const uint32_t tag = KT<K>::tag_of(key);
    for (int i = 0; i < kMaxProbe; i++) {
        K *b = table + bucket_of(h, i, nb) * S;
        K s[S];
        KT<K>::bucket(b, s);
        probes++;
#pragma unroll
        for (int j = 0; j < S; j++)
            if (KT<K>::eq(s[j], key)) return 0;
#pragma unroll
        for (int j = 0; j < S; j++) {
            // a torn slot is being filled: the CAS fails and returns the key
            if (KT<K>::empty(s[j], tag) || KT<K>::torn(s[j], tag)) {
                K old = KT<K>::cas(b + j, s[j], key);
                if (KT<K>::eq(old, s[j])) return 1;
                if (KT<K>::eq(old, key)) return 0;
            }
        }
    }
    return 2;
}

// ------------------------------------------------ placement with eviction
//
// A key whose 32 probe buckets were all full when it was inserted is appended to
// an overflow list; when the level's inserts are done (no lookup or insert runs
// any more) the list is placed.  A warp places one key X: its probe sequence is
// scanned again (X may have been placed meanwhile by a duplicate entry, or a
// slot freed, on the single-warp path); then, if the sequence is full, an
// occupant W whose own sequence has a free slot after W's position is moved
// there and X takes W's slot; if no occupant has one, an occupant is displaced
// anyway and placed the same way in turn, for at most kEvictDepth moves.
// Every move is a CAS from the contents just read, and a slot only ever changes
// from free to a key or from one key to another, so every slot that was
// occupied stays occupied: "every slot before a key's position is occupied"
// holds throughout and lookups stay exact.  Moves go forward (W's slot is taken
// before W is placed again), so no key is ever stored twice; a key that cannot
// be placed within kEvictDepth moves is reported as GPX_ERR_TABLE_FULL.  Reads
// are atomic (a 128-bit slot may change from one key to another while another
// warp places its keys).

template <class K> __device__ __forceinline__ K read_slot(K *p) {
    if (sizeof(K) <= 8) return KT<K>::load(p);
    const K z{};
    return KT<K>::cas(p, z, z); // compares with zero, writes zero only over zero: an atomic read
}

template <class K> __device__ __forceinline__ K shfl_key(const K &k, int src) {
    K o;
    if constexpr (sizeof(K) == 4) {
        o.v = __shfl_sync(kFull, k.v, src);
    } else if constexpr (sizeof(K) == 8) {
        o.v = __shfl_sync(kFull, k.v, src);
    } else {
        o.lo = __shfl_sync(kFull, k.lo, src);
        o.hi = __shfl_sync(kFull, k.hi, src);
    }
    return o;
}

// Place warp-uniform key x with eviction (all 32 lanes call it; kMaxProbe == 32,
// one probe bucket per lane).  Returns 0 if x was present, 1 if it was placed,
// 2 if a key could not be placed.  `moves` counts displaced keys (lane 0).
template <class K>
__device__ int place_warp(K *table, unsigned long long nb, K x, unsigned long long seed, uint32_t lane,
                          unsigned long long &moves) {
    static_assert(kMaxProbe == 32, "one probe bucket per lane");
    constexpr int S = KT<K>::kSlots;
    int depth = 0; // keys displaced so far; x is the key now looking for a slot
    for (int round = 0; round < 64; round++) { // each round returns, goes one move deeper or retries a lost race
        const uint64_t hx = KT<K>::hash(x, seed);
        const uint32_t tag = KT<K>::tag_of(x);
        const unsigned long long bx = bucket_of(hx, (int)lane, nb);
        K v[S];
        bool has = false;
        int fre = -1;
#pragma unroll
        for (int j = 0; j < S; j++) {
            v[j] = read_slot<K>(table + bx * S + j);
            if (KT<K>::eq(v[j], x)) has = true;
            if (fre < 0 && KT<K>::empty(v[j], tag)) fre = j;
        }
        if (__any_sync(kFull, has)) return depth ? 1 : 0; // (a displaced key is never found: stored once)
        const uint32_t fm = __ballot_sync(kFull, fre >= 0);
        if (fm) { // the first free slot in probe order
            const int L = __ffs(fm) - 1;
            int ok = 0;
            if ((int)lane == L) ok = KT<K>::eq(KT<K>::cas(table + bx * S + fre, v[fre], x), v[fre]);
            if (__shfl_sync(kFull, ok, L)) return 1;
            continue; // another placement took it: read again
        }
        if (depth >= kEvictDepth) return 2;
        // Full sequence.  Occupants in probe order, one at a time, each checked by
        // the whole warp for a free slot later in its own sequence.
        int step = 0; // 1: x placed, its occupant w is next (one move deeper); 2: lost a race
        for (int o = 0; o < 32 * S && !step; o++) {
            const int ob = o / S, oj = o % S;
            const unsigned long long bo = __shfl_sync(kFull, bx, ob);
            K w = v[0];
#pragma unroll
            for (int j = 0; j < S; j++) {
                const K t = shfl_key<K>(v[j], ob);
                if (j == oj) w = t;
            }
            const unsigned long long bw = bucket_of(KT<K>::hash(w, seed), (int)lane, nb);
            const uint32_t at = __ballot_sync(kFull, bw == bo); // w sits at its first visit of bo
            if (!at) continue;
            const int iw = __ffs(at) - 1;
            int fw = -1;
            K u[S];
#pragma unroll
            for (int j = 0; j < S; j++) u[j] = K{};
            if ((int)lane > iw) {
#pragma unroll
                for (int j = 0; j < S; j++) {
                    u[j] = read_slot<K>(table + bw * S + j);
                    if (fw < 0 && KT<K>::empty(u[j], tag)) fw = j;
                }
            }
            const uint32_t wm = __ballot_sync(kFull, fw >= 0);
            if (!wm) continue;
            // x takes w's slot first, then w the free slot: never two copies of w
            int ok = 0;
            if ((int)lane == ob) ok = KT<K>::eq(KT<K>::cas(table + bo * S + oj, w, x), w);
            if (!__shfl_sync(kFull, ok, ob)) {
                step = 2;
                break;
            }
            if (lane == 0) moves++;
            const int L = __ffs(wm) - 1;
            int ok2 = 0;
            if ((int)lane == L) ok2 = KT<K>::eq(KT<K>::cas(table + bw * S + fw, u[fw], w), u[fw]);
            if (__shfl_sync(kFull, ok2, L)) return 1;
            x = w; // lost the free slot: place w next
            depth++;
            step = 1;
        }
        if (step) continue;
        // No occupant has a free slot later in its sequence: displace a seeded one
        // anyway and place it next.
        const int o = (int)(mix64(hx + (uint64_t)depth) % (uint64_t)(32 * S));
        const int ob = o / S, oj = o % S;
        const unsigned long long bo = __shfl_sync(kFull, bx, ob);
        K w = v[0];
#pragma unroll
        for (int j = 0; j < S; j++) {
            const K t = shfl_key<K>(v[j], ob);
            if (j == oj) w = t;
        }
        int ok = 0;
        if ((int)lane == ob) ok = KT<K>::eq(KT<K>::cas(table + bo * S + oj, w, x), w);
        if (__shfl_sync(kFull, ok, ob)) {
            if (lane == 0) moves++;
            x = w;
            depth++;
        }
    }
    return 2; // kept losing races (bounded: the run reports a full table)
}

// Place the overflow list of a quiescent table with one warp, entry by entry
// (a later duplicate of a key finds it placed); new keys are appended to the
// store.  Used where a single warp closes a level (the many-network kernel).
template <class K>
__device__ void place_list_warp(K *table, unsigned long long nb, K *store, uint32_t *label,
                                unsigned long long store_cap, const K *overflow, unsigned long long n, Ctrl *c,
                                unsigned long long seed, uint32_t lane) {
    unsigned long long moves = 0, placed = 0;
    for (unsigned long long k = 0; k < n; k++) {
        const K x = KT<K>::load(overflow + k);
        const int r = place_warp<K>(table, nb, x, seed, lane, moves);
        if (r == 2) {
            if (lane == 0) set_error(c, GPX_ERR_TABLE_FULL);
            break;
        }
        if (r == 1 && lane == 0) {
            const unsigned long long idx = c->store_count++;
            if (idx < store_cap) {
                store[idx] = x;
                if (label) label[idx] = 0; // its inserting move is not kept: nothing is pruned from it
            } else {
                set_error(c, GPX_ERR_STORE_FULL);
            }
            placed++;
        }
    }
    if (lane == 0) {
        atomicAdd(&c->inserts, placed);
        atomicAdd(&c->evictions, moves);
        atomicAdd(&c->overflowed, n);
    }
    __syncwarp();
}

// The first overflow entry of key x (index k) wins a claim; a later entry of the
// same key (two threads inserted one new state while its sequence was full)
// finds the claim and is skipped, so each distinct key is placed once.
// Entries are {epoch, index} pairs; an entry of an older epoch is free.
template <class K>
__device__ bool claim_overflow(unsigned long long *claim, unsigned long long cap, unsigned long long epoch,
                               const K *overflow, unsigned long long k, const K &x, uint64_t h) {
    const unsigned long long mask = cap - 1;
    for (unsigned long long i = 0; i < cap; i++) {
        const unsigned long long pos = 2 + 2 * ((h + i) & mask); // [0, 2): the epoch counter
        unsigned long long olo, ohi;
        cas128(claim + pos, 0ull, 0ull, 0ull, 0ull, olo, ohi); // atomic read
        for (int tries = 0; tries < 64; tries++) {
            if (olo == epoch) break;
            unsigned long long nlo, nhi;
            cas128(claim + pos, olo, ohi, epoch, k, nlo, nhi);
            if (nlo == olo && nhi == ohi) return true; // claimed
            olo = nlo;
            ohi = nhi;
        }
        if (olo != epoch) return true; // unreachable in practice: behave as the first entry
        if (KT<K>::eq(KT<K>::load(overflow + ohi), x)) return ohi == k;
    }
    return true;
}

// Lookup in a table no one writes to during the call (the decide pass of the
// cycle proviso): an empty slot on the probe path means the key is absent.
template <class K>
__device__ __forceinline__ bool find_key(K *table, unsigned long long nb, const K &key, uint64_t h,
                                         unsigned int &probes) {
    constexpr int S = KT<K>::kSlots;
    const uint32_t tag = KT<K>::tag_of(key);
    for (int i = 0; i < kMaxProbe; i++) {
        K *b = table + bucket_of(h, i, nb) * S;
        K s[S];
        KT<K>::bucket(b, s);
        probes++;
#pragma unroll
        for (int j = 0; j < S; j++) {
            K v = s[j];
            if (KT<K>::torn(v, tag)) v = KT<K>::cas(b + j, v, v); // atomic re-read; the slot is complete
            if (KT<K>::eq(v, key)) return true;
            if (KT<K>::empty(v, tag)) return false;
        }
    }
    return false;
}

// --------------------------------------------------------- per-warp scratch

constexpr int kStage = 64; // new states staged per warp before one store append
constexpr uint32_t kRuleQueue = 64; // (pair, rule) items queued per warp in phase A

template <class K, int MODE> struct WarpScratch {
    static constexpr int kPairs = (MODE == MODE_PLAIN) ? kPairMax : kPairMaxPor;
    static constexpr int kPor = (MODE == MODE_PLAIN) ? 1 : kPairs;
    K keys[32];                  // the batch's source states
    K stage[kStage];             // new states waiting to be appended to the store
    uint32_t appl[kPairs];       // per pair: applicable rules among those it leads (bit r)
    uint32_t pre[kPairs + 1];    // per pair: successor count, then its exclusive prefix sum
    uint32_t en[32];             // per state: some transition enabled
    uint32_t cl0[kPor];          // per pair: static POR cluster
    uint32_t clo[kPor];          // per pair: cluster closure
    uint32_t nw[kPor];           // per pair: successors not yet visited (decide pass, for the log)
    uint16_t cand[kPor];         // learned proposal / log: the pairs whose closure is scored
    // POR modes, while successors are materialised (clo is dead then): the pair
    // of each successor index, when the batch has at most kOwners successors.
    // (Plain mode keeps the binary search: a 64-entry table of its own measured
    // 3% slower on the pruned config-2 kernel.)
    static constexpr uint32_t kOwners = (MODE == MODE_PLAIN) ? 0u : 4u * kPor;
    __device__ uint8_t *owner() { return reinterpret_cast<uint8_t *>(clo); }
    __device__ const uint8_t *owner() const { return reinterpret_cast<const uint8_t *>(clo); }
    static constexpr int kSrc = (MODE == MODE_PLAIN) ? 1 : 32; // per-state arrays of the POR modes
    static constexpr int kLab = (MODE == MODE_PLAIN) ? 32 : 1; // ... and of plain mode
    uint32_t prov[kSrc], sel[32], best[kSrc], vmask[kSrc];
    unsigned long long lbest[kSrc]; // learned proposal: (sortable score, popcount, process)
    uint32_t lab[kLab];                        // label of each source state
    uint32_t slab[kLab == 1 ? 1 : kStage];     // labels of the staged new states
    uint16_t ritem[kRuleQueue];                // queued (pair << 5 | rule) items of phase A
};

struct WarpStats {
    unsigned int lookups, probes, inserts, expanded, ilookups;
    unsigned int violation;
    unsigned int pruned;
};

// Model accessors over the device layout (gpx_model.h).  The array bases are
// resolved once; a process's bit field and record base come from one packed word.
struct MView {
    const uint32_t *w;
    uint32_t n;
    const uint32_t *recs, *ltgt_, *sent_, *stgt_, *rules_, *lrule_;
    __device__ void init(const uint32_t *m) {
        w = m;
        n = m[H_NPROCS];
        recs = m + m[H_OFF_RECS];
        ltgt_ = m + m[H_OFF_LTGT];
        sent_ = m + m[H_OFF_SENT];
        stgt_ = m + m[H_OFF_STGT];
        rules_ = m + m[H_OFF_RULES];
        lrule_ = m + m[H_OFF_LRULE];
    }
    __device__ uint32_t pd(uint32_t p) const { return w[H_PDESC + p]; }
    static __device__ uint32_t fb_of(uint32_t d) { return d & 127u; }
    static __device__ uint32_t bs_of(uint32_t d) { return (d >> 7) & 31u; }
    __device__ const uint32_t *rec_of(uint32_t d, uint32_t s) const { return recs + ((d >> 12) + s) * kRecWords; }
    __device__ uint32_t fb(uint32_t p) const { return fb_of(pd(p)); }
    __device__ uint32_t bs(uint32_t p) const { return bs_of(pd(p)); }
    __device__ const uint32_t *rec(uint32_t p, uint32_t s) const { return rec_of(pd(p), s); }
    __device__ uint32_t ltgt(uint32_t i) const { return ltgt_[i]; }
    __device__ uint32_t stgt(uint32_t i) const { return stgt_[i]; }
    __device__ uint32_t lrule(uint32_t i) const { return lrule_[i]; }
    __device__ uint32_t rmask(uint32_t k) const { return rules_[2 * k]; }
    __device__ uint32_t ract(uint32_t k) const { return rules_[2 * k + 1]; }
    // synchronising group of (p, s) for action a: {action, toff, tcnt, has1} or null
    __device__ const uint32_t *group(const uint32_t *rec, uint32_t a) const {
        const uint32_t *g = sent_ + rec[R_SOFF] * 4;
        for (uint32_t i = 0; i < rec[R_SCNT]; i++, g += 4) {
            if (g[0] == a) return g;
            if (g[0] > a) break;
        }
        return nullptr;
    }
    // local state of process p in `key` and its record
    template <class K> __device__ const uint32_t *state_rec(const K &key, uint32_t p, uint32_t &s) const {
        uint32_t d = pd(p);
        s = KT<K>::get(key, fb_of(d), bs_of(d));
        return rec_of(d, s);
    }
};

static __device__ __forceinline__ unsigned int vload(const unsigned int *p) { return *(volatile const unsigned int *)p; }
static __device__ __forceinline__ unsigned long long vload(const unsigned long long *p) {
    return *(volatile const unsigned long long *)p;
}

// Spin (with back-off) until *word differs from `old`, for at most timeout_ns.
// Returns false when the limit ran out: every device-side wait here ends.
static __device__ __forceinline__ bool wait_change(const unsigned int *word, unsigned int old, unsigned long long timeout_ns,
                                                   unsigned int max_sleep_ns = 1024) {
    uint64_t t0 = globaltimer();
    unsigned int ns = 32;
    while (vload(word) == old) {
        __nanosleep(ns);
        if (ns < max_sleep_ns) ns <<= 1;
        if (globaltimer() - t0 > timeout_ns) return false;
    }
    return true;
}

// ------------------------------------------- learned cluster proposal helpers

// Bucket of a (process, local state) pair among the 32 hashed one-hot features.
static __host__ __device__ __forceinline__ uint32_t por_hash_bucket(uint32_t p, uint32_t s) {
    uint32_t h = (p * 0x9E3779B1u) ^ (s * 0x85EBCA77u);
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    return h >> 27;
}

// d = c + sum_i a_i * b_i over the 4 bytes, a signed, b unsigned (exact).
static __device__ __forceinline__ int dp4a_su(uint32_t a, uint32_t b, int c) {
    int d;
    asm("dp4a.s32.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

// Round a non-negative float to bfloat16 precision, to nearest, ties to even.
static __host__ __device__ __forceinline__ float bf16_round(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    memcpy(&f, &u, 4);
    return f;
}

// MLP score of one candidate (features packed 4 per word, GPX_POR_FEATURES = 40).
static __device__ float por_mlp_score(const gpx_por_model *m, const uint32_t (&xw)[10]) {
    float out = 0.0f;
    for (int k = 0; k < GPX_POR_HIDDEN; k++) {
        const uint32_t *row = (const uint32_t *)m->w1[k];
        int acc = 0;
#pragma unroll
        for (int j = 0; j < 10; j++) acc = dp4a_su(__ldg(row + j), xw[j], acc);
        float h = fmaf((float)acc, __ldg(&m->s1[k]), __ldg(&m->b1[k]));
        h = h > 0.0f ? h : 0.0f;
        h = bf16_round(h);
        out = fmaf((float)m->w2[k], h, out);
    }
    return fmaf(out, m->s2, m->b2);
}

// Order-preserving map of a float to an unsigned key.
static __device__ __forceinline__ uint32_t float_key(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// ------------------------------------------------------------- the kernel

// WIDE: the explore kernel's wide batches -- phase A queues rule items across
// chunks, and POR modes tabulate each successor's pair.  The many-network
// kernel's small claims do neither: each lane evaluates its own pair's rules
// and successors find their pair by binary search, which keeps every claim's
// latency short.
template <class K, int MODE, bool WIDE = true> struct Explorer {
    const Params &P;
    MView M;
    WarpScratch<K, MODE> &ws;
    K *table;
    K *store;
    uint32_t lane;
    uint32_t lanemask_lt;
    uint32_t shead, scount; // staged new states (warp-uniform)
    WarpStats st;
    bool safety, deadlock;

    __device__ Explorer(const Params &p, const uint32_t *model, WarpScratch<K, MODE> &w)
        : P(p), ws(w), table((K *)p.table), store((K *)p.store) {
        M.init(model);
        lane = threadIdx.x & 31;
        lanemask_lt = (1u << lane) - 1u;
        shead = scount = 0;
        st = WarpStats{0, 0, 0, 0, 0, 0, 0};
        safety = P.property == GPX_PROP_SAFETY;
        deadlock = P.property == GPX_PROP_DEADLOCK;
    }

    // Successors of rule k from `key`: the product of the participants' targets.
    __device__ uint32_t product_size(const K &key, uint32_t mask, uint32_t act) const {
        uint32_t psz = 1, rest = mask;
        while (rest) {
            uint32_t q = __ffs(rest) - 1;
            rest &= rest - 1;
            uint32_t sq;
            psz *= M.group(M.state_rec(key, q, sq), act)[2];
        }
        return psz;
    }

    // Append `cnt` (<= 32) staged new states to the store with one atomic.
    __device__ void stage_flush(uint32_t cnt) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&P.ctrl->store_count, (unsigned long long)cnt);
        base = __shfl_sync(kFull, base, 0);
        if (lane < cnt) {
            unsigned long long idx = base + lane;
            if (idx < P.store_cap) {
                store[idx] = ws.stage[(shead + lane) % kStage];
                if (MODE == MODE_PLAIN && P.label) P.label[idx] = ws.slab[(shead + lane) % kStage];
            } else
                set_error(P.ctrl, GPX_ERR_STORE_FULL);
        }
        shead = (shead + cnt) % kStage;
        scount -= cnt;
        __syncwarp();
    }

    // Successor number t of the batch (ws.pre holds the per-pair prefix): the
    // pair's local targets first, then the products of the rules it leads.
    __device__ void materialise(uint32_t t, uint32_t npairs, bool filter, bool owned, K &out, uint32_t &og,
                                uint32_t &omask) const {
        const uint32_t n = M.n;
        uint32_t lo = 0, hi = npairs;
        if (owned) {
            lo = ws.owner()[t];
        } else {
            while (hi - lo > 1) {
                uint32_t mid = (lo + hi) >> 1;
                if (ws.pre[mid] <= t) lo = mid;
                else hi = mid;
            }
        }
        uint32_t sub = t - ws.pre[lo];
        og = lo / n;
        uint32_t p = lo - og * n;
        K key = ws.keys[og];
        const uint32_t dp = M.pd(p);
        const uint32_t *rec = M.rec_of(dp, KT<K>::get(key, MView::fb_of(dp), MView::bs_of(dp)));
        // plain mode: sel holds the processes whose local moves are not pruned
        uint32_t lcnt = ((MODE != MODE_PLAIN && !filter) || (ws.sel[og] >> p & 1u)) ? rec[R_LCNT] : 0u;
        out = key;
        omask = 0;
        if (sub < lcnt) {
            KT<K>::set(out, MView::fb_of(dp), MView::bs_of(dp), M.ltgt(rec[R_LOFF] + sub));
            omask = 1u << p;
            return;
        }
        sub -= lcnt;
        uint32_t a = ws.appl[lo], roff = rec[R_ROFF];
        while (a) {
            uint32_t r = __ffs(a) - 1;
            a &= a - 1;
            uint32_t k = M.lrule(roff + r), mask = M.rmask(k), act = M.ract(k);
            uint32_t psz = product_size(key, mask, act);
            if (sub >= psz) {
                sub -= psz;
                continue;
            }
            uint32_t rest = mask;
            while (rest) {
                uint32_t q = __ffs(rest) - 1;
                rest &= rest - 1;
                const uint32_t dq = M.pd(q);
                const uint32_t *grp = M.group(M.rec_of(dq, KT<K>::get(key, MView::fb_of(dq), MView::bs_of(dq))), act);
                uint32_t tc = grp[2], d = sub % tc;
                sub /= tc;
                KT<K>::set(out, MView::fb_of(dq), MView::bs_of(dq), M.stgt(grp[1] + d));
            }
            omask = mask;
            return;
        }
    }

    // Plain mode: is pair (g, p) below the lowest participant of the move that
    // first inserted state g (its local moves, and its rules disjoint from that
    // move, are pruned)?
    __device__ bool pruned_below(uint32_t g, uint32_t p) const {
        if (MODE != MODE_PLAIN) return false;
        const uint32_t lab = ws.lab[g];
        return lab && p < (uint32_t)(__ffs(lab) - 1);
    }

    // Rule number r among those pair i leads: applicable when every member has
    // its action enabled; its successors (the product of the members' targets)
    // are added to the pair's count unless pruned.
    __device__ void eval_rule(uint32_t i, uint32_t r, bool check) {
        const uint32_t g = i / M.n, p = i - g * M.n;
        const K key = ws.keys[g];
        uint32_t s;
        eval_rule(i, g, p, key, M.state_rec(key, p, s), r, check);
    }

    // ... for pair i = (state g, process p) whose key and record are at hand
    __device__ void eval_rule(uint32_t i, uint32_t g, uint32_t p, const K &key, const uint32_t *rec, uint32_t r,
                              bool check) {
        const uint32_t n = M.n;
        const uint32_t k = M.lrule(rec[R_ROFF] + r);
        const uint32_t mask = M.rmask(k), act = M.ract(k);
        // expand pass of the cycle proviso (no checks): rules inside the chosen cluster only
        if (MODE == MODE_PROVISO && !check && (mask & ws.sel[g]) != mask) return;
        bool hit1 = false;
        uint32_t rest = mask, psz = 1;
        while (rest) {
            const uint32_t q = __ffs(rest) - 1;
            rest &= rest - 1;
            uint32_t sq;
            const uint32_t *grp = M.group(q == p ? rec : M.state_rec(key, q, sq), act);
            if (!grp) return;
            psz *= grp[2];
            if (q == n - 1 && (grp[3] & 1u)) hit1 = true;
        }
        ws.en[g] = 1;
        if (MODE == MODE_POR) atomicOr(&ws.prov[g], mask);
        if (pruned_below(g, p) && (mask & ws.lab[g]) == 0) {
            st.pruned += psz;
        } else {
            atomicOr(&ws.appl[i], 1u << r);
            atomicAdd(&ws.pre[i], psz);
        }
        if (safety && check && hit1) st.violation = 1;
    }

    // Expand a batch of B states store[first .. first+B); the next `ahead`
    // states of the warp's claim are fetched into L2 meanwhile.
    __device__ void batch(unsigned long long first, uint32_t B, unsigned long long lvl_off, bool decide,
                          uint32_t ahead) {
        const uint32_t n = M.n;
        if (lane < ahead) {
            prefetch_l2(store + first + B + lane);
            if (MODE == MODE_PLAIN && P.label) prefetch_l2(P.label + first + B + lane);
        }
        if (lane < B) {
            ws.keys[lane] = KT<K>::load(store + first + lane);
            ws.en[lane] = 0;
            ws.sel[lane] = kFull;
            if (MODE != MODE_PLAIN) {
                ws.prov[lane] = 0;
                ws.best[lane] = kFull;
                ws.vmask[lane] = 0;
                ws.lbest[lane] = ~0ull;
                // expand pass of the cycle proviso: the cluster the decide pass chose
                if (MODE == MODE_PROVISO && !decide) ws.sel[lane] = __ldcg(P.sel + lvl_off + lane);
            } else {
                // commuting-move pruning: local moves of processes below the
                // label's lowest participant are generated from another state
                const uint32_t lab = P.label ? __ldcg(P.label + first + lane) : 0u;
                ws.lab[lane] = lab;
                if (lab) ws.sel[lane] = ~((1u << (__ffs(lab) - 1)) - 1u);
            }
        }
        __syncwarp();
        const uint32_t npairs = B * n;
        const bool check = (MODE != MODE_PROVISO) || decide;
        const bool filter = (MODE == MODE_POR) || (MODE == MODE_PROVISO && !decide);

        // A: enabledness, applicable rules, successor counts, static clusters,
        //    safety on moves into monitor state 1 (GPUexplore.cu:927-935, 1063-1069).
        //    Local moves per (state, process) pair; the rules a pair leads are
        //    queued as (pair, rule) items and evaluated 32 at a time, one per
        //    lane, instead of by the few lanes whose pair has rules.
        uint32_t rhead = 0, rcount = 0; // rule-item queue (warp-uniform)
        const uint32_t q32 = 32u / n, r32 = 32u - q32 * n;
        uint32_t g = lane / n, p = lane - g * n; // pair i = g * n + p, stepped by 32
        for (uint32_t base = 0; base < npairs; base += 32) {
            const uint32_t i = base + lane;
            uint32_t rcnt = 0;
            if (MODE == MODE_PROVISO && !decide && i < npairs && !(ws.sel[g] >> p & 1u)) {
                // expand pass of the cycle proviso: processes outside the chosen
                // cluster make no move (enabledness was checked in the decide pass)
                ws.appl[i] = 0;
                ws.pre[i] = 0;
            } else if (i < npairs) {
                K key = ws.keys[g];
                uint32_t s;
                const uint32_t *rec = M.state_rec(key, p, s);
                const uint32_t lcnt = rec[R_LCNT];
                rcnt = rec[R_RCNT];
                // Commuting-move pruning (plain mode).  The source was first
                // inserted by a move with participants `lab`.  A move led by a
                // process below lab's lowest participant and disjoint from lab
                // commutes with it: its successor also follows from the other
                // order, through a state of this same level with a higher-led
                // move, so it is not generated here.  Enabledness and the safety
                // check see every move.
                const bool below = pruned_below(g, p);
                ws.appl[i] = 0;
                ws.pre[i] = below ? 0u : lcnt;
                if (below) st.pruned += lcnt;
                if (MODE != MODE_PLAIN) {
                    // clusters feed the selection: the single POR pass, or the decide pass
                    if (MODE == MODE_POR || decide)
                        ws.cl0[i] = P.por_kind == POR_STUBBORN ? stubborn_cluster(key, p, rec) : rec[R_CL0];
                    ws.nw[i] = 0;
                }
                if (lcnt) {
                    ws.en[g] = 1;
                    if (MODE == MODE_POR) atomicOr(&ws.prov[g], 1u << p);
                }
                if (safety && check && p == n - 1 && (rec[R_FLAGS] & 1u)) st.violation = 1;
                if (!WIDE)
                    for (uint32_t x = 0; x < rcnt; x++) eval_rule(i, g, p, key, rec, x, check);
            }
            g += q32;
            p += r32;
            if (p >= n) {
                p -= n;
                g++;
            }
            if (!WIDE) continue;
            uint32_t incl = rcnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(kFull, incl, o);
                if (lane >= (uint32_t)o) incl += y;
            }
            const uint32_t T = __shfl_sync(kFull, incl, 31);
            if (!T) continue;
            if (rcount + T <= kRuleQueue) {
                for (uint32_t x = 0, at = rhead + rcount + incl - rcnt; x < rcnt; x++)
                    ws.ritem[(at + x) % kRuleQueue] = (uint16_t)((i << 5) | x);
                rcount += T;
                while (rcount >= 32) {
                    __syncwarp();
                    const uint32_t it = ws.ritem[(rhead + lane) % kRuleQueue];
                    __syncwarp();
                    eval_rule(it >> 5, it & 31u, check);
                    rhead = (rhead + 32) % kRuleQueue;
                    rcount -= 32;
                }
            } else {
                // more items than the queue holds: this chunk's lanes evaluate their own
                for (uint32_t x = 0; x < rcnt; x++) eval_rule(i, x, check);
            }
        }
        if (rcount) {
            __syncwarp();
            const uint32_t it = ws.ritem[(rhead + lane) % kRuleQueue];
            __syncwarp();
            if (lane < rcount) eval_rule(it >> 5, it & 31u, check);
        }
        __syncwarp();
        if (deadlock && check && lane < B && ws.en[lane] == 0) st.violation = 1;
        if (check && lane < B) st.expanded++;

        // B: the cluster each state expands (POR); without the cycle proviso the
        //    proviso bits are plain enabledness (GPUexplore.cu:1395-1397)
        if (MODE == MODE_POR) select_clusters(B, false);
        if (MODE == MODE_POR) {
            // successors of transitions inside the cluster only (GPUexplore.cu:1409, 1541);
            // the cycle proviso's expand pass applied its cluster in step A
            for (uint32_t i = lane; i < npairs; i += 32) {
                uint32_t g = i / n, p = i - g * n;
                uint32_t sel = ws.sel[g];
                K key = ws.keys[g];
                uint32_t sp;
                const uint32_t *rec = M.state_rec(key, p, sp);
                uint32_t cnt = (sel >> p & 1u) ? rec[R_LCNT] : 0u;
                uint32_t a = ws.appl[i], keep = 0, roff = rec[R_ROFF];
                while (a) {
                    uint32_t r = __ffs(a) - 1;
                    a &= a - 1;
                    uint32_t k = M.lrule(roff + r), mask = M.rmask(k);
                    if ((mask & sel) != mask) continue;
                    keep |= 1u << r;
                    cnt += product_size(key, mask, M.ract(k));
                }
                ws.appl[i] = keep;
                ws.pre[i] = cnt;
            }
            __syncwarp();
        }

        // exclusive prefix sum of the per-pair successor counts
        uint32_t carry = 0;
        for (uint32_t base = 0; base < npairs; base += 32) {
            uint32_t i = base + lane;
            uint32_t v = i < npairs ? ws.pre[i] : 0u, incl = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(kFull, incl, o);
                if (lane >= (uint32_t)o) incl += y;
            }
            if (i < npairs) ws.pre[i] = carry + incl - v;
            carry += __shfl_sync(kFull, incl, 31);
        }
        if (lane == 0) ws.pre[npairs] = carry;
        __syncwarp();
        // POR modes: the pair of every successor index, written once, instead of
        // a binary search over the prefix sums per successor
        const bool owned = WIDE && MODE != MODE_PLAIN && carry <= WarpScratch<K, MODE>::kOwners;
        if (owned) {
            for (uint32_t i = lane; i < npairs; i += 32)
                for (uint32_t t = ws.pre[i], e = ws.pre[i + 1]; t < e; t++) ws.owner()[t] = (uint8_t)i;
            __syncwarp();
        }

        // C: one successor per lane per round, materialised by index, then looked up
        for (uint32_t t0 = 0; t0 < carry; t0 += 32) {
            uint32_t t = t0 + lane;
            bool valid = t < carry;
            K out;
            uint32_t og = 0, omask = 0;
            if (valid) materialise(t, npairs, filter, owned, out, og, omask);
            if (MODE == MODE_PROVISO && decide) {
                if (valid) {
                    st.lookups++;
                    // cycle proviso: a successor satisfies it unless it is an explored
                    // ("OLD") state -- every state in the table during this pass
                    if (!find_key<K>(table, P.nbuckets, out, KT<K>::hash(out, P.seed), st.probes)) {
                        atomicOr(&ws.prov[og], omask);
                        if (P.log) atomicAdd(&ws.nw[og * M.n + (__ffs(omask) - 1)], 1u);
                    }
                }
                continue;
            }
            int res = -1;
            if (valid) {
                st.lookups++;
                st.ilookups++;
                res = find_or_insert<K>(table, P.nbuckets, out, KT<K>::hash(out, P.seed), st.probes);
                if (res == 2) { // full probe sequence: placed with eviction when the level closes
                    unsigned long long k = atomicAdd(&P.ctrl->overflow_count, 1ull);
                    if (k < P.overflow_cap)
                        ((K *)P.overflow)[k] = out;
                    else
                        set_error(P.ctrl, GPX_ERR_TABLE_FULL);
                }
            }
            uint32_t ins = __ballot_sync(kFull, res == 1);
            if (ins) {
                if (res == 1) {
                    const uint32_t pos = (shead + scount + __popc(ins & lanemask_lt)) % kStage;
                    ws.stage[pos] = out;
                    if (MODE == MODE_PLAIN) ws.slab[pos] = omask;
                    st.inserts++;
                }
                scount += __popc(ins);
                __syncwarp();
                if (scount >= 32) stage_flush(32);
            }
        }

        if (MODE == MODE_PROVISO && decide) {
            __syncwarp();
            select_clusters(B, true);
            if (lane < B) P.sel[lvl_off + lane] = ws.sel[lane];
        }
        __syncwarp();
    }

    // Successors generated by pair i's process (its local targets and the rules it
    // leads); `prefix` when ws.pre already holds the exclusive prefix sum.
    __device__ uint32_t pair_succ(uint32_t i, bool prefix) const { return prefix ? ws.pre[i + 1] - ws.pre[i] : ws.pre[i]; }

    // State-dependent cluster of process p (stubborn sets): {p}, and for every
    // rule containing p of an action p has enabled, all its members if the rule
    // is enabled, else only its lowest member without the action -- a necessary
    // enabling process that must move before the rule can fire.  A subset of the
    // static cluster (which takes every such rule whole).
    __device__ uint32_t stubborn_cluster(const K &key, uint32_t p, const uint32_t *rec) const {
        uint32_t cl = 1u << p;
        const uint32_t nr = M.w[H_NRULES];
        const uint32_t *g = M.sent_ + rec[R_SOFF] * 4;
        for (uint32_t j = 0; j < rec[R_SCNT]; j++, g += 4) {
            const uint32_t a = g[0];
            for (uint32_t k = g[3] >> 1; k < nr && M.ract(k) == a; k++) {
                const uint32_t mask = M.rmask(k);
                if (!(mask >> p & 1u)) continue;
                uint32_t lack = 0, rest = mask & ~(1u << p);
                while (rest) {
                    const uint32_t q = __ffs(rest) - 1;
                    rest &= rest - 1;
                    uint32_t sq;
                    if (!M.group(M.state_rec(key, q, sq), a)) {
                        lack = 1u << q;
                        break;
                    }
                }
                cl |= lack ? lack : mask;
            }
        }
        return cl;
    }

    // Features of candidate closure C of state g (GPX_POR_FEATURES small integers,
    // packed 4 per word): see include/gpx.h.
    __device__ void cluster_features(uint32_t g, uint32_t C, bool prefix, uint32_t (&xw)[10], uint32_t &succ) const {
        const uint32_t n = M.n;
        const K key = ws.keys[g];
        uint32_t x[GPX_POR_FEATURES];
#pragma unroll
        for (int j = 0; j < GPX_POR_FEATURES; j++) x[j] = 0;
        uint32_t lt = 0, sc = 0, deg = 0, rl = 0;
        uint32_t rest = C;
        while (rest) {
            uint32_t q = __ffs(rest) - 1;
            rest &= rest - 1;
            uint32_t sq = KT<K>::get(key, M.fb(q), M.bs(q));
            lt += M.rec(q, sq)[R_LCNT];
            sc += pair_succ(g * n + q, prefix);
            deg += __popc(ws.cl0[g * n + q]);
            rl += __popc(ws.appl[g * n + q]);
            x[8 + por_hash_bucket(q, sq)]++;
        }
        succ = sc;
        x[0] = __popc(C);
        x[1] = lt < 255 ? lt : 255;
        x[2] = sc < 255 ? sc : 255;
        x[3] = deg < 255 ? deg : 255;
        x[4] = __popc(C & ws.prov[g]);
        x[5] = n;
        x[6] = rl < 255 ? rl : 255;
        x[7] = 1;
#pragma unroll
        for (int w = 0; w < 10; w++)
            xw[w] = x[4 * w] | (x[4 * w + 1] << 8) | (x[4 * w + 2] << 16) | (x[4 * w + 3] << 24);
    }

    // Cluster per state (GPUexplore.cu:1633-1672): close each process's cluster
    // (its own bit dropped when its proviso fails), keep closures with a member
    // whose proviso holds, take the smallest (ties: lowest process; default: all)
    // -- or, with the learned proposal, the lowest-scoring valid closure after the
    // proposal passes the same checks.  ws.prov holds the proviso bits.
    __device__ void select_clusters(uint32_t B, bool prefix) {
        if (MODE == MODE_PLAIN) return;
        const uint32_t n = M.n;
        __syncwarp();
        const uint32_t npairs = B * n;
        for (uint32_t i = lane; i < npairs; i += 32) {
            uint32_t g = i / n, p = i - g * n;
            uint32_t prov = ws.prov[g];
            const uint32_t *cl = ws.cl0 + g * n;
            uint32_t cp = (prov >> p & 1u) ? cl[p] : (cl[p] & ~(1u << p));
            uint32_t closure = cp, todo = cp, valid = 0;
            while (todo) {
                uint32_t q = __ffs(todo) - 1;
                todo &= ~(1u << q);
                uint32_t cq = (prov >> q & 1u) ? cl[q] : (cl[q] & ~(1u << q));
                valid |= (cq >> q) & 1u;
                todo |= cq & ~closure & ~(1u << q);
                closure |= cq;
            }
            ws.clo[i] = closure;
            // ample: only a single process whose enabled transitions involve no other process
            if (valid && closure && (P.por_kind != POR_AMPLE || __popc(closure) == 1)) {
                atomicMin(&ws.best[g], ((uint32_t)__popc(closure) << 5) | p);
                atomicOr(&ws.vmask[g], 1u << p);
            }
        }
        __syncwarp();
        const bool learn = P.learned && P.por_model;
        const bool logging = (MODE == MODE_PROVISO) && P.log && prefix;
        if (learn || logging) {
            // compact the candidates (one per distinct valid closure of a state) so
            // that every lane of a round scores one: a round costs a whole MLP
            uint32_t ncand = 0;
            for (uint32_t base = 0; base < npairs; base += 32) {
                const uint32_t i = base + lane;
                bool cand = false;
                if (i < npairs) {
                    const uint32_t g = i / n, p = i - g * n;
                    if (ws.vmask[g] >> p & 1u) {
                        const uint32_t C = ws.clo[i];
                        cand = true;
                        for (uint32_t q = 0; q < p; q++)
                            if ((ws.vmask[g] >> q & 1u) && ws.clo[g * n + q] == C) cand = false;
                    }
                }
                const uint32_t m = __ballot_sync(kFull, cand);
                if (cand) ws.cand[ncand + __popc(m & lanemask_lt)] = (uint16_t)i;
                ncand += __popc(m);
            }
            __syncwarp();
            for (uint32_t c = lane; c < ncand; c += 32) {
                const uint32_t i = ws.cand[c];
                const uint32_t g = i / n, p = i - g * n;
                const uint32_t C = ws.clo[i];
                uint32_t xw[10], succ = 0;
                cluster_features(g, C, prefix, xw, succ);
                if (learn) {
                    float sc = por_mlp_score(P.por_model, xw);
                    if (isfinite(sc))
                        atomicMin(&ws.lbest[g], ((unsigned long long)float_key(sc) << 32) |
                                                     (((uint32_t)__popc(C) << 5) | p));
                }
                if (logging) {
                    uint32_t tag = (uint32_t)KT<K>::hash(ws.keys[g], 0x5BD1E995ull);
                    if (P.log_every && (tag % P.log_every) == 0) {
                        unsigned long long slot = atomicAdd(P.log_count, 1ull);
                        if (slot < P.log_cap) {
                            gpx_por_log_row *row = P.log + slot;
                            uint32_t nwsum = 0, rest = C;
                            while (rest) {
                                uint32_t q = __ffs(rest) - 1;
                                rest &= rest - 1;
                                nwsum += ws.nw[g * n + q];
                            }
                            for (int w = 0; w < 10; w++) ((uint32_t *)row->x)[w] = xw[w];
                            row->succ = succ;
                            row->new_succ = nwsum;
                            row->state_tag = tag;
                            row->popc = (uint8_t)__popc(C);
                            uint32_t b = ws.best[g];
                            row->cample_choice = (b != kFull && ws.clo[g * n + (b & 31u)] == C) ? 1 : 0;
                            row->pad[0] = row->pad[1] = 0;
                        }
                    }
                }
            }
            __syncwarp();
        }
        if (lane < B) {
            uint32_t b = ws.best[lane];
            uint32_t all = (n == 32) ? kFull : ((1u << n) - 1u);
            uint32_t sel = (b == kFull || (b >> 5) >= n) ? all : ws.clo[lane * n + (b & 31u)];
            if (learn && ws.lbest[lane] != ~0ull) {
                // re-check the proposal: non-empty, closed under the members'
                // clusters, and some member's proviso holds; else plain cample
                uint32_t C = ws.clo[lane * n + (uint32_t)(ws.lbest[lane] & 31u)];
                uint32_t prov = ws.prov[lane], rest = C;
                bool closed = C != 0, some = (C & prov) != 0;
                while (rest) {
                    uint32_t q = __ffs(rest) - 1;
                    rest &= rest - 1;
                    uint32_t cq = ws.cl0[lane * n + q];
                    if (!(prov >> q & 1u)) cq &= ~(1u << q);
                    if (cq & ~C) closed = false;
                }
                if (closed && some) sel = C;
            }
            ws.sel[lane] = sel;
        }
        __syncwarp();
    }

    // End of a level: append the staged new states and report a violation.
    // The counters stay in registers (flushed by flush_counters) unless a lane
    // nears the range of its 32-bit counts.
    __device__ void flush_level() {
        if (scount) stage_flush(scount);
        if (__any_sync(kFull, st.violation) && lane == 0) atomicOr(&P.ctrl->violation, 1u);
        st.violation = 0;
        if (__any_sync(kFull, st.probes > (1u << 30) || st.lookups > (1u << 30) || st.pruned > (1u << 30)))
            flush_counters();
    }

    __device__ void flush_counters() {
        Ctrl *c = P.ctrl;
        unsigned long long v[6] = {st.lookups, st.probes, st.inserts, st.expanded, st.ilookups, st.pruned};
#pragma unroll
        for (int k = 0; k < 6; k++)
            for (int o = 16; o; o >>= 1) v[k] += __shfl_xor_sync(kFull, v[k], o);
        if (lane == 0) {
            if (v[0]) atomicAdd(&c->lookups, v[0]);
            if (v[1]) atomicAdd(&c->probes, v[1]);
            if (v[2]) atomicAdd(&c->inserts, v[2]);
            if (v[3]) atomicAdd(&c->expanded, v[3]);
            if (v[4]) atomicAdd(&c->inserts_lookups, v[4]);
            if (v[5]) atomicAdd(&c->pruned, v[5]);
        }
        st = WarpStats{0, 0, 0, 0, 0, st.violation, 0};
    }

    __device__ void flush_stats() {
        flush_level();
        flush_counters();
    }
};

} // namespace gpx
