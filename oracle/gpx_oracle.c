/*
 * gpx_oracle.c -- CPU oracle for GPUexplore-style state-space exploration.
 *
 * TEST INFRASTRUCTURE ONLY.  This program is the checker for the GPU path: only
 * the tests, the package smoke check and the CPU-baseline leg of the benchmark
 * run it.  The product (libgpx) never links, loads or calls it.
 *
 * What it computes: a plain level-synchronous BFS over the gpf semantics of the
 * reference (GPUexplore/src/GPUexplore.cu, cited below as G:<line>), from the
 * all-zero initial state, with
 *   - per-level new-state counts (level 0 = the initial state),
 *   - the deadlock verdict (an expanded state with no enabled transition,
 *     G:1134-1151) and the safety verdict (a generated successor whose last
 *     process is in local state 1, G:927-935, G:1063-1069),
 *   - optional cluster-based ample-set ("cample") partial-order reduction with
 *     or without the cycle proviso (G:1345-1675), restated deterministically:
 *     the proviso of a successor is "not in the visited set as it stood at the
 *     start of the level" (the reference's "not found-and-OLD in the global
 *     table", G:454-493, G:1418-1428),
 *   - exploration stops at the end of the level in which a violation is found
 *     (the reference stops at the end of the launch, G:2122-2126) or at the end
 *     of the level at which the visited count reaches --max-states.
 *
 * Semantics are the intended ones of G:904-1122: a local entry's targets each
 * give a successor; a synchronising action a fires rule r iff every process in
 * r has at least one a-entry, and then yields the Cartesian product of the
 * participants' a-targets.
 *
 * Parallel form: each level is processed in chunks; threads generate successors
 * into per-(thread, shard) buffers, then each thread owns one shard of the
 * visited set and inserts that shard's successors.  The result (the visited
 * set, per-level counts and verdicts) does not depend on the thread count.
 *
 * Parity status: unpinned by the reference, which ships no tests, fixtures,
 * golden vectors or CPU path.  This oracle is pinned against hand-derived known
 * answers and an independent enumerator over the generators' abstract models
 * (tests/golden).
 */
#define _GNU_SOURCE
#include <inttypes.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { PROP_NONE = 0, PROP_DEADLOCK = 1, PROP_SAFETY = 2, PROP_LIVENESS = 3 };

/* ---------------------------------------------------------------- gpf model */

typedef struct {
    uint32_t liveness, nr_procs, bits_act, proc_nrstates, bits_statevector;
    uint32_t *firstbit, *bits_state;
    uint32_t nbits_offset, max_buf_ints;
    uint32_t *proc_offsets_start, *proc_offsets;
    uint32_t nr_trans, *proc_trans;
    uint32_t nbits_syncbits_offset, nr_syncbits_offsets, *syncbits_offsets;
    uint32_t nr_syncbits, *syncbits;
    uint32_t W; /* words per state vector key: ceil(firstbit[nr_procs] / 32) */
} gpf_t;

typedef struct {
    FILE *f;
    int ok;
} reader_t;

/* One integer per line with atoi semantics, kept as unsigned 32-bit (G:1888-1982). */
static uint32_t next_int(reader_t *r) {
    char buf[256];
    if (!fgets(buf, sizeof buf, r->f)) {
        r->ok = 0;
        return 0;
    }
    return (uint32_t)strtoll(buf, NULL, 10);
}

static uint32_t *read_array(reader_t *r, uint32_t n) {
    uint32_t *a = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
    for (uint32_t i = 0; i < n; i++) a[i] = next_int(r);
    return a;
}

/* gpf loader: field order of G:1885-1987. */
static int gpf_load(const char *path, gpf_t *m) {
    reader_t r = {fopen(path, "r"), 1};
    if (!r.f) return -1;
    memset(m, 0, sizeof *m);
    m->liveness = next_int(&r);
    m->nr_procs = next_int(&r);
    m->bits_act = next_int(&r);
    m->proc_nrstates = next_int(&r);
    m->bits_statevector = next_int(&r);
    if (!r.ok || m->nr_procs < 1 || m->nr_procs > 31 || m->bits_act < 1 || m->bits_act > 30) {
        fclose(r.f);
        return -2;
    }
    m->firstbit = read_array(&r, m->nr_procs + 1);
    m->bits_state = read_array(&r, m->nr_procs);
    m->nbits_offset = next_int(&r);
    m->max_buf_ints = next_int(&r);
    m->proc_offsets_start = read_array(&r, m->nr_procs + 1);
    m->proc_offsets = read_array(&r, m->proc_offsets_start[m->nr_procs]);
    m->nr_trans = next_int(&r);
    m->proc_trans = read_array(&r, m->nr_trans);
    m->nbits_syncbits_offset = next_int(&r);
    m->nr_syncbits_offsets = next_int(&r);
    m->syncbits_offsets = read_array(&r, m->nr_syncbits_offsets);
    m->nr_syncbits = next_int(&r);
    m->syncbits = read_array(&r, m->nr_syncbits);
    fclose(r.f);
    if (!r.ok) return -2;
    if (m->nbits_offset < 1 || m->nbits_offset > 31 || m->nbits_syncbits_offset < 1 ||
        m->nbits_syncbits_offset > 31)
        return -2;
    for (uint32_t p = 0; p < m->nr_procs; p++)
        if (m->firstbit[p + 1] - m->firstbit[p] != m->bits_state[p] || m->bits_state[p] < 1 ||
            m->bits_state[p] > 31 - m->bits_act)
            return -2;
    uint32_t bits = m->firstbit[m->nr_procs];
    m->W = bits ? (bits + 31) / 32 : 1;
    return 0;
}

/* ------------------------------------------------------------ field access */

/* Bits [lo, lo+len) of a field-packed word array, fields from bit 0 (G:156, G:160-161). */
static inline uint32_t packed_field(const uint32_t *words, uint32_t i, uint32_t nbits) {
    uint32_t per = 32 / nbits;
    return (words[i / per] >> ((i % per) * nbits)) & ((1u << nbits) - 1u);
}

/* Local state of process p: bits [firstbit[p], firstbit[p+1]), may straddle two
 * words (GETSTATEVECTORSTATE, G:162-169). */
static inline uint32_t get_local(const gpf_t *m, const uint32_t *v, uint32_t p) {
    uint32_t lo = m->firstbit[p], w = m->bits_state[p];
    uint64_t x = v[lo / 32];
    if ((lo % 32) + w > 32) x |= (uint64_t)v[lo / 32 + 1] << 32;
    return (uint32_t)((x >> (lo % 32)) & ((1ull << w) - 1));
}

/* Overwrite process p's local state (SETSTATEVECTORSTATE, G:170-178). */
static inline void set_local(const gpf_t *m, uint32_t *v, uint32_t p, uint32_t x) {
    uint32_t lo = m->firstbit[p], w = m->bits_state[p];
    uint64_t mask = ((1ull << w) - 1) << (lo % 32);
    uint64_t cur = v[lo / 32];
    int two = (lo % 32) + w > 32;
    if (two) cur |= (uint64_t)v[lo / 32 + 1] << 32;
    cur = (cur & ~mask) | (((uint64_t)x << (lo % 32)) & mask);
    v[lo / 32] = (uint32_t)cur;
    if (two) v[lo / 32 + 1] = (uint32_t)(cur >> 32);
}

/* Transition range [o1, o2) of process p in local state s (G:883-898). */
static inline void trans_range(const gpf_t *m, uint32_t p, uint32_t s, uint32_t *o1, uint32_t *o2) {
    const uint32_t *base = m->proc_offsets + m->proc_offsets_start[p];
    *o1 = packed_field(base, s, m->nbits_offset);
    *o2 = packed_field(base, s + 1, m->nbits_offset);
}

static inline uint32_t entry_is_sync(uint32_t e) { return e & 1u; }                     /* G:158 */
static inline uint32_t entry_action(const gpf_t *m, uint32_t e) {                       /* G:157 */
    return (e >> 1) & ((1u << m->bits_act) - 1u);
}
static inline uint32_t entry_slots(const gpf_t *m, uint32_t p) {                        /* G:143 */
    return (31 - m->bits_act) / m->bits_state[p];
}
/* Slot i of an entry: target+1, 0 = unused (G:159). */
static inline uint32_t entry_slot(const gpf_t *m, uint32_t e, uint32_t i, uint32_t p) {
    uint32_t w = m->bits_state[p];
    return (e >> (1 + m->bits_act + i * w)) & ((1u << w) - 1u);
}

/* Rule range of action a in syncbits: fields a and a+1 (G:998-1009). */
static inline void rule_range(const gpf_t *m, uint32_t a, uint32_t *o1, uint32_t *o2) {
    uint32_t per = 32 / m->nbits_syncbits_offset;
    if ((a + 1) / per >= m->nr_syncbits_offsets) {
        *o1 = *o2 = 0;
        return;
    }
    *o1 = packed_field(m->syncbits_offsets, a, m->nbits_syncbits_offset);
    *o2 = packed_field(m->syncbits_offsets, a + 1, m->nbits_syncbits_offset);
}

/* ------------------------------------------------------- successor relation */

#define MAXP 32
#define MAXT 64 /* targets per (process, action) kept for the product */
#define MAXA 16 /* distinct synchronising actions per (process, local state) */

static void capacity_exceeded(const char *what) {
    fprintf(stderr, "ERROR: oracle capacity exceeded: %s\n", what);
    exit(2);
}

typedef struct {
    uint32_t act;
    uint32_t n;
    uint32_t t[MAXT];
} actset_t;

typedef struct {
    /* per process: local targets and synchronising (action, targets) groups */
    uint32_t nlocal[MAXP];
    uint32_t local[MAXP][MAXT];
    uint32_t nacts[MAXP];
    actset_t acts[MAXP][MAXA];
} expand_t;

/* Collect p's transitions from local state s: local entries' targets, and
 * synchronising targets grouped by action (entries of one action are adjacent,
 * G:955-978, G:1437-1456). */
static void collect(const gpf_t *m, const uint32_t *v, expand_t *x) {
    for (uint32_t p = 0; p < m->nr_procs; p++) {
        uint32_t s = get_local(m, v, p), o1, o2;
        trans_range(m, p, s, &o1, &o2);
        x->nlocal[p] = 0;
        x->nacts[p] = 0;
        uint32_t ns = entry_slots(m, p);
        for (uint32_t k = o1; k < o2 && k < m->nr_trans; k++) {
            uint32_t e = m->proc_trans[k];
            if (!entry_is_sync(e)) {
                for (uint32_t i = 0; i < ns; i++) { /* G:921-943 */
                    uint32_t t = entry_slot(m, e, i, p);
                    if (!t) break;
                    if (x->nlocal[p] == MAXT) capacity_exceeded("local targets");
                    x->local[p][x->nlocal[p]++] = t - 1;
                }
            } else {
                uint32_t a = entry_action(m, e);
                actset_t *g = x->nacts[p] ? &x->acts[p][x->nacts[p] - 1] : NULL;
                if (!g || g->act != a) {
                    if (x->nacts[p] == MAXA) capacity_exceeded("synchronising actions per state");
                    g = &x->acts[p][x->nacts[p]++];
                    g->act = a;
                    g->n = 0;
                }
                for (uint32_t i = 0; i < ns; i++) {
                    uint32_t t = entry_slot(m, e, i, p);
                    if (!t) break;
                    if (g->n == MAXT) capacity_exceeded("targets per action");
                    g->t[g->n++] = t - 1;
                }
            }
        }
    }
}

static const actset_t *find_act(const expand_t *x, uint32_t p, uint32_t a) {
    for (uint32_t i = 0; i < x->nacts[p]; i++)
        if (x->acts[p][i].act == a) return &x->acts[p][i];
    return NULL;
}

/* A generated successor with the set of processes whose transitions produced it:
 * a local move of p carries mask 1<<p, a synchronisation carries its rule mask. */
typedef struct {
    uint32_t mask;
    uint32_t is_local;
} origin_t;

typedef void (*emit_fn)(void *ctx, const uint32_t *succ, origin_t o);

/* When set (per thread), counts each applicable rule at its lowest member. */
static __thread uint32_t *g_rules_led = NULL;

/* Enumerate every successor of v (G:904-949 local, G:954-1122 synchronising). */
static int expand_all(const gpf_t *m, const uint32_t *v, const expand_t *x, emit_fn emit, void *ctx) {
    uint32_t succ[16];
    int enabled = 0;
    const uint32_t n = m->nr_procs, W = m->W;
    for (uint32_t p = 0; p < n; p++) {
        for (uint32_t j = 0; j < x->nlocal[p]; j++) {
            memcpy(succ, v, W * 4);
            set_local(m, succ, p, x->local[p][j]);
            origin_t o = {1u << p, 1};
            emit(ctx, succ, o);
            enabled = 1;
        }
    }
    /* synchronising actions in ascending order, each once (the minimum-action
     * merge of G:979-995 visits every action enabled in some process) */
    uint32_t done[MAXP * MAXA];
    uint32_t ndone = 0;
    for (uint32_t p = 0; p < n; p++) {
        for (uint32_t i = 0; i < x->nacts[p]; i++) {
            uint32_t a = x->acts[p][i].act, seen = 0;
            for (uint32_t d = 0; d < ndone; d++)
                if (done[d] == a) seen = 1;
            if (seen) continue;
            done[ndone++] = a;
            uint32_t en = 0; /* processes with an a-entry: proc_enabled, G:995 / G:1463 */
            for (uint32_t q = 0; q < n; q++)
                if (find_act(x, q, a)) en |= 1u << q;
            uint32_t r1, r2;
            rule_range(m, a, &r1, &r2);
            uint32_t per = 32 / n;
            for (uint32_t w = r1; w < r2 && w < m->nr_syncbits; w++) {
                for (uint32_t f = 0; f < per; f++) {
                    uint32_t rule = (m->syncbits[w] >> (f * n)) & ((n == 32) ? 0xFFFFFFFFu : ((1u << n) - 1u));
                    if (!rule || (rule & en) != rule) continue; /* G:1016, G:1488 */
                    enabled = 1;
                    if (g_rules_led) g_rules_led[__builtin_ctz(rule)]++;
                    /* Cartesian product over the participants' a-targets (G:1030-1119) */
                    const actset_t *g[MAXP];
                    uint32_t parts[MAXP], np = 0, idx[MAXP];
                    for (uint32_t q = 0; q < n; q++)
                        if (rule >> q & 1u) {
                            parts[np] = q;
                            g[np] = find_act(x, q, a);
                            idx[np] = 0;
                            np++;
                        }
                    for (;;) {
                        memcpy(succ, v, W * 4);
                        for (uint32_t k = 0; k < np; k++) set_local(m, succ, parts[k], g[k]->t[idx[k]]);
                        origin_t o = {rule, 0};
                        emit(ctx, succ, o);
                        uint32_t k = 0;
                        while (k < np && ++idx[k] == g[k]->n) idx[k++] = 0;
                        if (k == np) break;
                    }
                }
            }
        }
    }
    return enabled;
}

/* ------------------------------------------------- learned cluster proposal */

/* The proposal MLP in the byte layout of gpx_por_model (include/gpx.h): int8
 * w1[64][40], float s1[64], float b1[64], int8 w2[64], float s2, b2.  The
 * selection below restates the GPU's exactly: integer features, an exact integer
 * layer-1 sum, fmaf in the same order, bfloat16 round-to-nearest-even. */
#define PF 40
#define PH 64
typedef struct {
    int8_t w1[PH][PF];
    float s1[PH];
    float b1[PH];
    int8_t w2[PH];
    float s2, b2;
} por_model_t;

static por_model_t *g_por_model = NULL;

static float bf16_round(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    memcpy(&f, &u, 4);
    return f;
}

static uint32_t por_hash_bucket(uint32_t p, uint32_t s) {
    uint32_t h = (p * 0x9E3779B1u) ^ (s * 0x85EBCA77u);
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    return h >> 27;
}

static float por_score(const por_model_t *m, const uint32_t *x) {
    float out = 0.0f;
    for (int k = 0; k < PH; k++) {
        int acc = 0;
        for (int j = 0; j < PF; j++) acc += (int)m->w1[k][j] * (int)x[j];
        float h = fmaf((float)acc, m->s1[k], m->b1[k]);
        h = h > 0.0f ? h : 0.0f;
        h = bf16_round(h);
        out = fmaf((float)m->w2[k], h, out);
    }
    return fmaf(out, m->s2, m->b2);
}

static uint32_t float_key(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

/* Static cluster of process p: {p} plus every rule containing p of an action
 * that p has enabled, whether or not the rule is applicable (G:1616-1624). */
static uint32_t static_cluster(const gpf_t *m, const expand_t *x, uint32_t p) {
    uint32_t c = 1u << p, n = m->nr_procs, per = 32 / n;
    for (uint32_t i = 0; i < x->nacts[p]; i++) {
        uint32_t r1, r2;
        rule_range(m, x->acts[p][i].act, &r1, &r2);
        for (uint32_t w = r1; w < r2 && w < m->nr_syncbits; w++)
            for (uint32_t f = 0; f < per; f++) {
                uint32_t rule = (m->syncbits[w] >> (f * n)) & ((1u << n) - 1u);
                if (rule >> p & 1u) c |= rule;
            }
    }
    return c;
}

/* Cluster selection from per-process clusters and proviso bits (G:1633-1672):
 * drop p's own bit if its proviso failed, close each process's cluster under the
 * cluster relation, keep closures with at least one member whose proviso held,
 * take the one with the fewest processes (ties: lowest process index); default
 * is every process (full expansion). */
typedef struct {
    uint32_t succ[MAXP];   /* successors each process leads (local targets + led rules' products) */
    uint32_t nlocal[MAXP]; /* local targets */
    uint32_t rules[MAXP];  /* applicable rules led */
    uint32_t s[MAXP];      /* local states */
} por_ctx_t;

/* Stubborn-set cluster of process p in state v: {p}, and for every rule
 * containing p of an action p has enabled, the rule's members if every member
 * has the action, else only its lowest member without it (a necessary enabling
 * process).  A subset of static_cluster. */
static uint32_t stubborn_cluster(const gpf_t *m, const expand_t *x, uint32_t p) {
    uint32_t c = 1u << p, n = m->nr_procs, per = 32 / n;
    for (uint32_t i = 0; i < x->nacts[p]; i++) {
        uint32_t a = x->acts[p][i].act, r1, r2;
        rule_range(m, a, &r1, &r2);
        for (uint32_t w = r1; w < r2 && w < m->nr_syncbits; w++)
            for (uint32_t f = 0; f < per; f++) {
                uint32_t rule = (m->syncbits[w] >> (f * n)) & ((1u << n) - 1u);
                if (!(rule >> p & 1u)) continue;
                uint32_t lack = 0;
                for (uint32_t q = 0; q < n && !lack; q++)
                    if ((rule >> q & 1u) && !find_act(x, q, a)) lack = 1u << q;
                c |= lack ? lack : rule;
            }
    }
    return c;
}

/* ample: only single-process closures qualify */
static int g_ample = 0;

static uint32_t select_cluster(uint32_t n, const uint32_t *cl, uint32_t prov, const por_ctx_t *pc) {
    uint32_t c[MAXP];
    for (uint32_t p = 0; p < n; p++) c[p] = (prov >> p & 1u) ? cl[p] : (cl[p] & ~(1u << p));
    uint32_t best = (n == 32) ? 0xFFFFFFFFu : ((1u << n) - 1u);
    uint32_t bestc = n;
    uint64_t lbest = ~0ull;
    uint32_t lsel = 0;
    for (uint32_t p = 0; p < n; p++) {
        uint32_t closure = c[p], todo = c[p], valid = 0;
        while (todo) {
            uint32_t i = (uint32_t)__builtin_ctz(todo);
            todo &= ~(1u << i);
            valid |= (c[i] >> i) & 1u;
            todo |= c[i] & ~closure & ~(1u << i);
            closure |= c[i];
        }
        if (valid && closure && (!g_ample || __builtin_popcount(closure) == 1) &&
            (uint32_t)__builtin_popcount(closure) < bestc) {
            bestc = (uint32_t)__builtin_popcount(closure);
            best = closure;
        }
        if (g_por_model && pc && valid && closure) {
            /* features of the candidate (the GPU's cluster_features) */
            uint32_t x[PF];
            memset(x, 0, sizeof x);
            uint32_t lt = 0, sc = 0, deg = 0, rl = 0;
            for (uint32_t q = 0; q < n; q++)
                if (closure >> q & 1u) {
                    lt += pc->nlocal[q];
                    sc += pc->succ[q];
                    deg += (uint32_t)__builtin_popcount(cl[q]);
                    rl += pc->rules[q];
                    x[8 + por_hash_bucket(q, pc->s[q])]++;
                }
            x[0] = (uint32_t)__builtin_popcount(closure);
            x[1] = lt < 255 ? lt : 255;
            x[2] = sc < 255 ? sc : 255;
            x[3] = deg < 255 ? deg : 255;
            x[4] = (uint32_t)__builtin_popcount(closure & prov);
            x[5] = n;
            x[6] = rl < 255 ? rl : 255;
            x[7] = 1;
            float sco = por_score(g_por_model, x);
            if (isfinite(sco)) {
                uint64_t key = ((uint64_t)float_key(sco) << 32) | (((uint32_t)__builtin_popcount(closure) << 5) | p);
                if (key < lbest) {
                    lbest = key;
                    lsel = closure;
                }
            }
        }
    }
    if (lbest != ~0ull) {
        /* re-check the proposal: non-empty, closed, a member whose proviso holds */
        int closed = lsel != 0, some = (lsel & prov) != 0;
        for (uint32_t q = 0; q < n; q++)
            if ((lsel >> q & 1u) && (c[q] & ~lsel)) closed = 0;
        if (closed && some) return lsel;
    }
    return best;
}

/* ---------------------------------------------------------------- hash sets */

static inline uint64_t mix64(uint64_t z) { /* SplitMix64 finaliser (Steele, Lea, Flood 2014) */
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Hash of a key; also the per-state term of the order-independent set hash. */
static inline uint64_t key_hash(const uint32_t *k, uint32_t W) {
    uint64_t h = 0x9E3779B97F4A7C15ull;
    for (uint32_t j = 0; j < W; j += 2) {
        uint64_t c = k[j];
        if (j + 1 < W) c |= (uint64_t)k[j + 1] << 32;
        h = mix64(h ^ c);
    }
    return h;
}

typedef struct {
    uint32_t *keys;
    uint8_t *used;
    uint64_t cap, n;
    uint32_t W;
} hset_t;

static void hset_init(hset_t *s, uint32_t W, uint64_t cap) {
    s->W = W;
    s->cap = cap;
    s->n = 0;
    s->keys = (uint32_t *)malloc(cap * W * 4);
    s->used = (uint8_t *)calloc(cap, 1);
}

static int hset_find(const hset_t *s, const uint32_t *k, uint64_t h) {
    uint64_t i = h & (s->cap - 1); /* the shard is chosen by the high bits */
    for (;;) {
        if (!s->used[i]) return 0;
        if (!memcmp(s->keys + i * s->W, k, s->W * 4)) return 1;
        i = (i + 1) & (s->cap - 1);
    }
}

static int hset_insert(hset_t *s, const uint32_t *k, uint64_t h);

static void hset_grow(hset_t *s) {
    hset_t t;
    hset_init(&t, s->W, s->cap * 2);
    for (uint64_t i = 0; i < s->cap; i++)
        if (s->used[i]) hset_insert(&t, s->keys + i * s->W, key_hash(s->keys + i * s->W, s->W));
    free(s->keys);
    free(s->used);
    *s = t;
}

static int hset_insert(hset_t *s, const uint32_t *k, uint64_t h) {
    if ((s->n + 1) * 2 > s->cap) hset_grow(s);
    uint64_t i = h & (s->cap - 1);
    for (;;) {
        if (!s->used[i]) {
            s->used[i] = 1;
            memcpy(s->keys + i * s->W, k, s->W * 4);
            s->n++;
            return 1;
        }
        if (!memcmp(s->keys + i * s->W, k, s->W * 4)) return 0;
        i = (i + 1) & (s->cap - 1);
    }
}

typedef struct {
    uint32_t *a;
    uint64_t n, cap;
} vec_t;

static inline void vec_push(vec_t *v, const uint32_t *k, uint32_t W) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 1024;
        v->a = (uint32_t *)realloc(v->a, v->cap * W * 4);
    }
    memcpy(v->a + v->n * W, k, W * 4);
    v->n++;
}

/* ------------------------------------------------------------------- search */

typedef struct {
    int property, por, proviso, threads;
    uint64_t max_states;
    const char *dump;
    int quiet;
} opts_t;

typedef struct {
    const gpf_t *m;
    const opts_t *o;
    hset_t *shards;
    uint32_t nshards;
    /* per-state scratch for POR */
    uint32_t prov;
    int safety_hit;
    int cycle; /* evaluating cycle-proviso lookups */
    /* successor sink */
    vec_t *out; /* [nshards] for the calling thread */
    uint32_t sel;
    uint64_t generated;
    por_ctx_t pc; /* per-process facts for the learned proposal */
} sctx_t;

static inline uint32_t shard_of(uint64_t h, uint32_t nshards) {
    return (uint32_t)(((h >> 32) * (uint64_t)nshards) >> 32);
}

static void check_safety(sctx_t *c, const uint32_t *succ) {
    /* G:927-935 / G:1063-1069: last process in local state 1 */
    if (c->o->property == PROP_SAFETY && get_local(c->m, succ, c->m->nr_procs - 1) == 1) c->safety_hit = 1;
}

/* Pass-1 sink: properties and (with the cycle proviso) proviso bits. */
static void emit_decide(void *ctx, const uint32_t *succ, origin_t o) {
    sctx_t *c = (sctx_t *)ctx;
    check_safety(c, succ);
    int sat = 1;
    if (c->cycle) {
        uint64_t h = key_hash(succ, c->m->W);
        sat = !hset_find(&c->shards[shard_of(h, c->nshards)], succ, h);
    }
    if (sat) c->prov |= o.mask; /* local: bit p; synchronisation: every member (G:1616-1624) */
    c->pc.succ[__builtin_ctz(o.mask)]++;    /* attributed to the lowest member, as the GPU's leader */
}

/* Pass-2 sink: keep successors of transitions inside the selected cluster
 * (G:1409, G:1541: local of p iff p in cluster, rule r iff r within cluster). */
static void emit_keep(void *ctx, const uint32_t *succ, origin_t o) {
    sctx_t *c = (sctx_t *)ctx;
    c->generated++;
    if ((o.mask & c->sel) != o.mask) return;
    uint64_t h = key_hash(succ, c->m->W);
    vec_push(&c->out[shard_of(h, c->nshards)], succ, c->m->W);
}

/* Without reduction: check the property and keep every successor in one pass. */
static void emit_plain(void *ctx, const uint32_t *succ, origin_t o) {
    sctx_t *c = (sctx_t *)ctx;
    (void)o;
    check_safety(c, succ);
    c->generated++;
    uint64_t h = key_hash(succ, c->m->W);
    vec_push(&c->out[shard_of(h, c->nshards)], succ, c->m->W);
}

typedef struct {
    uint64_t *level_counts;
    uint32_t nlevels;
    uint64_t states;
    uint64_t generated;
    int violation;
    int stopped; /* 0 done, 1 violation, 2 budget */
    uint64_t set_hash;
    double seconds;
    uint64_t live_states; /* states in accepting cyclic components (liveness) */
} result_t;

static int liveness_check(const gpf_t *m, hset_t *shards, uint32_t S, uint64_t *scc_states);

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + ts.tv_nsec * 1e-9;
}

/* Decide the cluster of one frontier state (POR) and check its properties. */
static uint32_t decide(sctx_t *c, const uint32_t *v, expand_t *x, int *deadlock) {
    const gpf_t *m = c->m;
    collect(m, v, x);
    c->prov = 0;
    memset(&c->pc, 0, sizeof c->pc);
    g_rules_led = c->pc.rules;
    int enabled = expand_all(m, v, x, emit_decide, c);
    g_rules_led = NULL;
    if (!enabled) *deadlock = 1;
    if (!c->o->por) return 0xFFFFFFFFu;
    uint32_t cl[MAXP];
    for (uint32_t p = 0; p < m->nr_procs; p++) {
        cl[p] = c->o->por == 4 ? stubborn_cluster(m, x, p) : static_cluster(m, x, p);
        c->pc.nlocal[p] = x->nlocal[p];
        c->pc.s[p] = get_local(m, v, p);
    }
    return select_cluster(m->nr_procs, cl, c->prov, c->o->por == 2 ? &c->pc : NULL);
}

static int run(const gpf_t *m, const opts_t *o, result_t *res) {
    const uint32_t W = m->W;
    int T = 1;
#ifdef _OPENMP
    T = o->threads > 0 ? o->threads : omp_get_max_threads();
    omp_set_dynamic(0); /* thread t owns shard t: every shard needs its thread */
    omp_set_num_threads(T);
#endif
    const uint32_t S = (uint32_t)T;
    hset_t *shards = (hset_t *)calloc(S, sizeof(hset_t));
    for (uint32_t j = 0; j < S; j++) hset_init(&shards[j], W, 1024);

    vec_t frontier = {0}, next = {0};
    vec_t *outs = (vec_t *)calloc((size_t)S * S, sizeof(vec_t));
    vec_t *nexts = (vec_t *)calloc(S, sizeof(vec_t));
    uint32_t *init = (uint32_t *)calloc(W, 4);
    uint64_t h0 = key_hash(init, W);
    hset_insert(&shards[shard_of(h0, S)], init, h0);
    vec_push(&frontier, init, W);
    uint64_t total = 1, generated = 0;
    uint64_t cap_levels = 1024;
    res->level_counts = (uint64_t *)malloc(cap_levels * 8);
    res->level_counts[0] = 1;
    res->nlevels = 1;
    res->violation = 0;
    res->stopped = 0;
    uint32_t *sel = NULL;
    uint64_t sel_cap = 0;
    const int need_pass1 = o->por && o->proviso;
    const uint64_t CHUNK = 1u << 16;
    FILE *dump = o->dump ? fopen(o->dump, "wb") : NULL;
    if (dump) fwrite(init, 4, W, dump);

    double t0 = now_s();
    while (frontier.n) {
        int violation = 0;
        if (need_pass1) {
            /* cycle proviso: decide every frontier state's cluster before any insert of
             * this level, so lookups see the visited set as of the level's start */
            if (frontier.n > sel_cap) {
                sel_cap = frontier.n;
                sel = (uint32_t *)realloc(sel, sel_cap * 4);
            }
#pragma omp parallel reduction(| : violation)
            {
                expand_t *x = (expand_t *)malloc(sizeof(expand_t));
                sctx_t c = {.m = m, .o = o, .shards = shards, .nshards = S, .cycle = 1}; /* the rest zero */
#pragma omp for schedule(dynamic, 256)
                for (int64_t i = 0; i < (int64_t)frontier.n; i++) {
                    int dl = 0;
                    c.safety_hit = 0;
                    sel[i] = decide(&c, frontier.a + i * W, x, &dl);
                    if ((dl && o->property == PROP_DEADLOCK) || c.safety_hit) violation = 1;
                }
                free(x);
            }
        }
        uint64_t level_new = 0;
        for (uint64_t base = 0; base < frontier.n; base += CHUNK) {
            uint64_t end = base + CHUNK < frontier.n ? base + CHUNK : frontier.n;
            uint64_t gen_chunk = 0;
#pragma omp parallel reduction(| : violation) reduction(+ : gen_chunk)
            {
                int t = 0;
#ifdef _OPENMP
                t = omp_get_thread_num();
#endif
                expand_t *x = (expand_t *)malloc(sizeof(expand_t));
                sctx_t c = {.m = m, .o = o, .shards = shards, .nshards = S, .out = outs + (size_t)t * S}; /* the rest zero */
#pragma omp for schedule(dynamic, 256)
                for (int64_t i = (int64_t)base; i < (int64_t)end; i++) {
                    const uint32_t *v = frontier.a + i * W;
                    if (!o->por) {
                        c.safety_hit = 0;
                        collect(m, v, x);
                        int en = expand_all(m, v, x, emit_plain, &c);
                        if ((!en && o->property == PROP_DEADLOCK) || c.safety_hit) violation = 1;
                        continue;
                    }
                    if (need_pass1) {
                        collect(m, v, x);
                        c.sel = sel[i];
                    } else {
                        int dl = 0;
                        c.safety_hit = 0;
                        c.sel = decide(&c, v, x, &dl);
                        if ((dl && o->property == PROP_DEADLOCK) || c.safety_hit) violation = 1;
                    }
                    expand_all(m, v, x, emit_keep, &c);
                }
                gen_chunk += c.generated;
                free(x);
#pragma omp barrier
                /* thread t owns shard t: insert every thread's successors for it */
                for (uint32_t s = 0; s < S; s++) {
                    vec_t *src = &outs[(size_t)s * S + t];
                    for (uint64_t k = 0; k < src->n; k++) {
                        const uint32_t *key = src->a + k * W;
                        uint64_t h = key_hash(key, W);
                        if (hset_insert(&shards[t], key, h)) vec_push(&nexts[t], key, W);
                    }
                    src->n = 0;
                }
            }
            generated += gen_chunk;
        }
        next.n = 0;
        for (uint32_t j = 0; j < S; j++) {
            for (uint64_t k = 0; k < nexts[j].n; k++) vec_push(&next, nexts[j].a + k * W, W);
            nexts[j].n = 0;
        }
        level_new = next.n;
        total += level_new;
        if (level_new) {
            if (res->nlevels == cap_levels) {
                cap_levels *= 2;
                res->level_counts = (uint64_t *)realloc(res->level_counts, cap_levels * 8);
            }
            res->level_counts[res->nlevels++] = level_new;
            if (dump) fwrite(next.a, 4, (size_t)next.n * W, dump);
        }
        vec_t tmp = frontier;
        frontier = next;
        next = tmp;
        if (violation) {
            res->violation = 1;
            res->stopped = 1;
            break;
        }
        if (o->max_states && total >= o->max_states && frontier.n) {
            res->stopped = 2;
            break;
        }
    }
    res->seconds = now_s() - t0;
    res->states = total;
    res->generated = generated;
    uint64_t sh = 0;
    for (uint32_t j = 0; j < S; j++)
        for (uint64_t i = 0; i < shards[j].cap; i++)
            if (shards[j].used[i]) sh += key_hash(shards[j].keys + i * W, W);
    res->set_hash = sh;
    res->live_states = 0;
    if (o->property == PROP_LIVENESS && !o->por && res->stopped == 0 && !res->violation) {
        if (liveness_check(m, shards, S, &res->live_states)) {
            res->violation = 1;
            res->stopped = 1;
        }
    }
    if (dump) fclose(dump);
    return 0;
}

/* --------------------------------------------------------------- liveness */

/* The gpf liveness flag (G:1888-1898) is parsed but never checked by the
 * reference.  Here it means: the last process is a Buchi automaton whose local
 * state 1 is accepting, and the property is violated iff some reachable cycle
 * contains an accepting state.  Checked after a complete exploration without
 * POR: the explicit graph of the visited set, Tarjan's strongly connected
 * components (iterative), and a component with an accepting state that holds
 * a cycle (more than one state, or a self-loop) is a violation. */
typedef struct {
    const gpf_t *m;
    const uint32_t *all;  /* N x W visited states */
    const int64_t *slot;  /* open-addressing index: slot -> state index or -1 */
    uint64_t mask;
    uint32_t *edges;
    uint64_t nedges, cap;
} graph_ctx_t;

static int64_t index_of(const graph_ctx_t *g, const uint32_t *k) {
    const uint32_t W = g->m->W;
    uint64_t i = key_hash(k, W) & g->mask;
    for (;;) {
        int64_t v = g->slot[i];
        if (v < 0) return -1;
        if (!memcmp(g->all + (uint64_t)v * W, k, W * 4)) return v;
        i = (i + 1) & g->mask;
    }
}

static void emit_edge(void *ctx, const uint32_t *succ, origin_t o) {
    (void)o;
    graph_ctx_t *g = (graph_ctx_t *)ctx;
    int64_t j = index_of(g, succ);
    if (j < 0) { /* every successor of a visited state was visited: the search was complete */
        fprintf(stderr, "ERROR: liveness check: successor outside the visited set\n");
        exit(1);
    }
    if (g->nedges == g->cap) {
        g->cap = g->cap ? 2 * g->cap : 1024;
        g->edges = (uint32_t *)realloc(g->edges, g->cap * 4);
    }
    g->edges[g->nedges++] = (uint32_t)j;
}

/* 1 when an accepting cycle exists; *scc_states = states in accepting cyclic components */
static int liveness_check(const gpf_t *m, hset_t *shards, uint32_t S, uint64_t *scc_states) {
    const uint32_t W = m->W, n = m->nr_procs;
    uint64_t N = 0;
    for (uint32_t j = 0; j < S; j++) N += shards[j].n;
    if (N >= 0xFFFFFFFFull) capacity_exceeded("states for the liveness check");
    uint32_t *all = (uint32_t *)malloc(N * W * 4);
    uint64_t k = 0;
    for (uint32_t j = 0; j < S; j++)
        for (uint64_t i = 0; i < shards[j].cap; i++)
            if (shards[j].used[i]) memcpy(all + (k++) * W, shards[j].keys + i * W, W * 4);
    uint64_t cap = 1;
    while (cap < 2 * N) cap <<= 1;
    int64_t *slot = (int64_t *)malloc(cap * 8);
    for (uint64_t i = 0; i < cap; i++) slot[i] = -1;
    for (uint64_t v = 0; v < N; v++) {
        uint64_t i = key_hash(all + v * W, W) & (cap - 1);
        while (slot[i] >= 0) i = (i + 1) & (cap - 1);
        slot[i] = (int64_t)v;
    }
    graph_ctx_t g = {m, all, slot, cap - 1, NULL, 0, 0};
    uint64_t *first = (uint64_t *)malloc((N + 1) * 8);
    expand_t *x = (expand_t *)malloc(sizeof(expand_t));
    for (uint64_t v = 0; v < N; v++) {
        first[v] = g.nedges;
        collect(m, all + v * W, x);
        expand_all(m, all + v * W, x, emit_edge, &g);
    }
    first[N] = g.nedges;
    free(x);
    /* Tarjan, iterative: index/low per state, an explicit DFS stack of (state, next edge) */
    uint32_t *idx = (uint32_t *)malloc(N * 4), *low = (uint32_t *)malloc(N * 4);
    uint8_t *on = (uint8_t *)calloc(N, 1);
    uint32_t *stk = (uint32_t *)malloc(N * 4), *dfs = (uint32_t *)malloc(N * 4);
    uint64_t *it = (uint64_t *)malloc(N * 8);
    for (uint64_t v = 0; v < N; v++) idx[v] = 0xFFFFFFFFu;
    uint32_t counter = 0;
    uint64_t sp = 0, dp = 0, found = 0;
    for (uint64_t r = 0; r < N; r++) {
        if (idx[r] != 0xFFFFFFFFu) continue;
        dfs[dp++] = (uint32_t)r;
        idx[r] = low[r] = counter++;
        it[r] = first[r];
        stk[sp++] = (uint32_t)r;
        on[r] = 1;
        while (dp) {
            uint32_t v = dfs[dp - 1];
            if (it[v] < first[v + 1]) {
                uint32_t w = g.edges[it[v]++];
                if (idx[w] == 0xFFFFFFFFu) {
                    idx[w] = low[w] = counter++;
                    it[w] = first[w];
                    stk[sp++] = w;
                    on[w] = 1;
                    dfs[dp++] = w;
                } else if (on[w] && idx[w] < low[v]) {
                    low[v] = idx[w];
                }
                continue;
            }
            dp--;
            if (dp && low[v] < low[dfs[dp - 1]]) low[dfs[dp - 1]] = low[v];
            if (low[v] != idx[v]) continue;
            /* v roots a component: pop it */
            uint64_t size = 0, acc = 0, self = 0, top = sp;
            uint32_t w;
            do {
                w = stk[--sp];
                on[w] = 0;
                size++;
                if (get_local(m, all + (uint64_t)w * W, n - 1) == 1) acc = 1;
            } while (w != v);
            if (size == 1)
                for (uint64_t e = first[v]; e < first[v + 1]; e++)
                    if (g.edges[e] == v) self = 1;
            if (acc && (size > 1 || self)) found += size;
            (void)top;
        }
    }
    *scc_states = found;
    free(all);
    free(slot);
    free(first);
    free(g.edges);
    free(idx);
    free(low);
    free(on);
    free(stk);
    free(dfs);
    free(it);
    return found > 0;
}

static void usage(void) {
    fprintf(stderr,
            "usage: gpx_oracle <model>[.gpf] [-d|-p] [--por|--ample|--stubborn] [--cycle-proviso] [--threads N]\n"
            "                  [--max-states N] [--dump-states FILE]\n");
}

int main(int argc, char **argv) {
    if (argc < 2) {
        usage();
        return 1;
    }
    opts_t o = {PROP_NONE, 0, 0, 1, 0, NULL, 0};
    char path[4096];
    size_t len = strlen(argv[1]);
    if (len > 4 && !strcmp(argv[1] + len - 4, ".gpf"))
        snprintf(path, sizeof path, "%s", argv[1]);
    else
        snprintf(path, sizeof path, "%s.gpf", argv[1]); /* G:1814-1815 */
    /* option semantics of G:1817-1883: -d turns the cycle proviso off, -p turns it on,
     * --cycle-proviso only counts when no property flag came before it */
    for (int i = 2; i < argc; i++) {
        if (!strcmp(argv[i], "-d")) {
            o.property = PROP_DEADLOCK;
            o.proviso = 0;
        } else if (!strcmp(argv[i], "-p")) {
            o.property = PROP_SAFETY;
            o.proviso = 1;
        } else if (!strcmp(argv[i], "--por-model") && i + 1 < argc) {
            FILE *pf = fopen(argv[++i], "rb");
            g_por_model = (por_model_t *)calloc(1, sizeof(por_model_t));
            if (!pf || fread(g_por_model, sizeof(por_model_t), 1, pf) != 1) {
                fprintf(stderr, "ERROR: cannot read POR model %s\n", argv[i]);
                return 1;
            }
            fclose(pf);
            o.por = 2;
        } else if (!strcmp(argv[i], "--por")) {
            if (!o.por) o.por = 1;
        } else if (!strcmp(argv[i], "--ample")) {
            o.por = 3;
            g_ample = 1;
        } else if (!strcmp(argv[i], "--stubborn")) {
            o.por = 4;
        } else if (!strcmp(argv[i], "--cycle-proviso")) {
            if (o.property == PROP_NONE) o.proviso = 1;
        } else if (!strcmp(argv[i], "--threads") && i + 1 < argc) {
            o.threads = atoi(argv[++i]);
        } else if (!strcmp(argv[i], "--max-states") && i + 1 < argc) {
            o.max_states = strtoull(argv[++i], NULL, 10);
        } else if (!strcmp(argv[i], "--dump-states") && i + 1 < argc) {
            o.dump = argv[++i];
        } else {
            fprintf(stderr, "ERROR: unrecognized option %s\n", argv[i]);
            usage();
            return 1;
        }
    }
    gpf_t m;
    int rc = gpf_load(path, &m);
    if (rc == -1) {
        fprintf(stderr, "ERROR: input network does not exist!\n"); /* G:1985 */
        return 1;
    }
    if (rc) {
        fprintf(stderr, "ERROR: malformed gpf file\n");
        return 1;
    }
    if (o.property == PROP_SAFETY && m.liveness == 1) o.property = PROP_LIVENESS; /* G:1888-1898 */
    if (m.bits_statevector + (uint32_t)o.por > 32u * 16u || m.W > 16) {
        fprintf(stderr, "ERROR: state vector too wide for the oracle\n");
        return 1;
    }
    if (o.property == PROP_LIVENESS && o.por) {
        fprintf(stderr, "ERROR: the liveness check needs the full state graph (no --por)\n");
        return 1;
    }
    result_t r;
    run(&m, &o, &r);
    int T = 1;
#ifdef _OPENMP
    T = o.threads > 0 ? o.threads : omp_get_max_threads();
#endif
    const char *verdict = "none";
    if (r.violation)
        verdict = o.property == PROP_DEADLOCK ? "deadlock" : (o.property == PROP_LIVENESS ? "liveness" : "safety");
    printf("{\"states\": %" PRIu64 ", \"levels\": [", r.states);
    for (uint32_t i = 0; i < r.nlevels; i++) printf("%s%" PRIu64, i ? ", " : "", r.level_counts[i]);
    printf("], \"verdict\": \"%s\", \"stopped\": \"%s\", \"generated\": %" PRIu64
           ", \"set_hash\": \"%016" PRIx64 "\", \"threads\": %d, \"seconds\": %.6f, \"words\": %u"
           ", \"live_states\": %" PRIu64 "}\n",
           verdict, r.stopped == 0 ? "done" : (r.stopped == 1 ? "violation" : "budget"), r.generated,
           r.set_hash, T, r.seconds, m.W, r.live_states);
    return 0;
}
