/*
 * gpx.h -- C ABI of libgpx, the GB300 (sm_103a) state-space explorer.
 *
 * The reference (GPUexplore) has no library API: its boundary is the process
 * level -- `GPUexplore <model> [options]`, a <model>.gpf file and stdout lines
 * (GPUexplore/src/GPUexplore.cu:1738-2188).  This header exposes that boundary
 * as plain C entry points (plain pointers and sizes, no C++ or torch types) so a
 * C, C++, Python (ctypes) or other FFI caller can drive the same exploration
 * in-process; the `gpuexplore` command-line tool is a thin client of it.
 *
 * Threading: a gpx_explorer is used by one host thread at a time.  Calls block
 * until the device work they start has finished.  One device per explorer.
 */
#ifndef GPX_H
#define GPX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPX_ABI_VERSION 4

/* Status codes.  They replace the reference's exit(1) paths. */
typedef enum {
    GPX_OK = 0,
    GPX_ERR_PARSE = 1,       /* missing or malformed gpf input (GPUexplore.cu:1984-1987) */
    GPX_ERR_NO_GPU = 2,      /* no CUDA device (GPUexplore.cu:1999-2003) */
    GPX_ERR_CUDA = 3,        /* a CUDA runtime call failed (CUDA_CHECK_RETURN, GPUexplore.cu:522-528) */
    GPX_ERR_TABLE_FULL = 4,  /* every probe bucket of a state was full ("problem with hash table",
                                contBFS == 2, GPUexplore.cu:1170-1173, 2164-2166) */
    GPX_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up (no reference counterpart) */
    GPX_ERR_INVALID = 6,     /* invalid argument */
    GPX_ERR_UNSUPPORTED = 7, /* model outside this build's limits (state vector > 126 bits,
                                > 31 processes) */
    GPX_ERR_STORE_FULL = 8,  /* the state store (the BFS queue of visited states) overflowed */
    GPX_ERR_NOMEM = 9        /* device or host allocation failed */
} gpx_status;

/* Property to check (PropertyStatus, GPUexplore.cu:27). */
typedef enum {
    GPX_PROP_NONE = 0,
    GPX_PROP_DEADLOCK = 1, /* -d */
    GPX_PROP_SAFETY = 2,   /* -p: last process reaches local state 1 */
    GPX_PROP_LIVENESS = 3  /* -p with gpf line 1 == 1: the reference parses it and checks nothing
                              (GPUexplore.cu:1888-1898); here an accepting cycle through local state 1 of
                              the last process is searched after a complete exploration without POR */
} gpx_property;

typedef enum {
    GPX_STOP_DONE = 0,      /* no unexplored states left */
    GPX_STOP_VIOLATION = 1, /* property violated; stopped at the end of that BFS level */
    GPX_STOP_BUDGET = 2,    /* max_states reached at the end of a level */
    GPX_STOP_ERROR = 3      /* see gpx_result.status */
} gpx_stop;

/* Options: the reference's command-line flags (GPUexplore.cu:1785-1883) plus
 * the controls this build adds.  Initialise with gpx_options_init(). */
typedef struct {
    uint32_t struct_size;   /* sizeof(gpx_options), set by gpx_options_init */
    int32_t blocks;         /* -b: blocks of the persistent kernel (0 = every SM, full occupancy) */
    int32_t threads;        /* -t: threads per block (0 = 256) */
    int32_t kernel_iters;   /* -k: BFS levels per kernel launch (0 = run to the end in one launch) */
    int32_t verbosity;      /* -v 0..3 (clamped to 3, GPUexplore.cu:1846-1848) */
    uint64_t q_words;       /* -q: hash-table size in 32-bit words (0 = half the free device memory) */
    int32_t por;            /* --por: 1 cluster-based ample sets (cample), 2 cample with the learned proposal,
                               3 single-process ample sets, 4 stubborn sets (necessary-enabling clusters) */
    int32_t cycle_proviso;  /* --cycle-proviso */
    int32_t property;       /* gpx_property */
    int32_t device;         /* CUDA device ordinal */
    uint64_t seed;          /* seed of the hash functions (does not affect any result) */
    uint64_t max_states;    /* stop at the end of the level that reaches this many states (0 = off) */
    uint64_t store_states;  /* capacity of the state store in states (0 = as many as table slots) */
    int32_t collect_states; /* copy the visited states back into gpx_result.states */
    int32_t bucket_bytes;   /* hash bucket size in bytes: 0 or 32 (one DRAM sector; other values are rejected) */
    int32_t launch_graph;   /* 1 (gpx_options_init): with verbosity 0, a run is one CUDA graph -- reset, init,
                               a device-side loop over the exploration launches (the -k relaunch loop),
                               set hash and read-back -- built once and replayed; 0: host-driven launches */
    int32_t prune_commuting; /* 1 (gpx_options_init), plain exploration by a gpx_explorer: a state does not
                                generate the successors of moves that commute with the move that first
                                inserted it and are led by a lower process -- a state of the same level
                                generates each of them -- so fewer lookups reach the table; the visited
                                set, level counts and verdicts are unchanged; 0: every successor */
    int32_t set_hash;       /* 1: fill gpx_result.set_hash (one extra pass over the state store after the
                               exploration, ~0.5 ms per 1.6e8 states: a check of the visited set against another
                               explorer); 0 (gpx_options_init): skip the pass, set_hash = 0 */
} gpx_options;

/* Result of one exploration.  Arrays are owned by the library: gpx_result_free. */
typedef struct {
    uint32_t struct_size;
    int32_t status;          /* gpx_status of the run */
    int32_t stopped;         /* gpx_stop */
    int32_t verdict;         /* gpx_property that was violated, or GPX_PROP_NONE */
    uint64_t states;         /* visited states ("nr. of states in hash table", GPUexplore.cu:2172) */
    uint32_t nlevels;        /* BFS levels discovered, level 0 = the initial state */
    uint64_t *level_counts;  /* new states per level [nlevels] */
    uint64_t transitions;    /* successor instances generated */
    uint64_t probes;         /* hash-bucket probes (lookups and inserts) */
    uint64_t launches;       /* kernel launches of the exploration loop */
    double explore_ms;       /* device time of the exploration (CUDA events) */
    double setup_ms;         /* host time spent on table reset and model upload */
    uint64_t set_hash;       /* order-independent hash of the visited set (sum of key hashes); 0 unless
                                gpx_options.set_hash */
    uint32_t key_words;      /* 32-bit words per state vector in `states_buf` */
    uint64_t table_count;    /* occupied hash-table slots, counted by a sweep like count_states
                                (GPUexplore.cu:687-704); filled when collect_states or verbosity >= 2 */
    uint64_t lookups;        /* successors looked up in the hash table */
    uint64_t expanded;       /* frontier states expanded */
    double kernel_ms;        /* device time of the exploration kernel launches only */
    uint32_t *states_buf;    /* visited states [states * key_words] in BFS order, when collected */
    uint64_t table_slots;    /* hash-table capacity in states */
    uint32_t slot_bytes;     /* bytes per hash-table slot (4, 8 or 16) */
    uint32_t blocks, threads;/* launch configuration that ran */
    uint64_t inserts;        /* states inserted into the hash table by the exploration kernels */
    uint64_t evictions;      /* stored states displaced within their probe sequence to make room */
    uint64_t h2d_bytes;      /* bytes this run copied host -> device (model uploads are counted by set_model) */
    uint64_t d2h_bytes;      /* bytes this run copied device -> host (without collect_states / -v output) */
    uint64_t live_states;    /* liveness: states left in the accepting-cycle fixpoint (0 = no accepting cycle) */
    double live_ms;          /* liveness: device time of the accepting-cycle check */
    uint64_t live_rounds;    /* liveness: frontier rounds (forward closure and peeling) of the check */
    uint32_t table_generation; /* 128-bit slots of a reusable explorer table (state vectors of 64..112
                                  bits): the generation (1..255) this run's keys carry; slots of other
                                  generations read as free, so only some runs clear the table; 0 for
                                  the untagged slot forms, which every run clears */
    int32_t table_cleared;   /* this run zeroed the hash table before it started */
    uint64_t pruned;         /* successors not generated by commuting-move pruning (gpx_options.prune_commuting);
                                with it, lookups/transitions/probes depend on which of a state's predecessors
                                inserted it first and vary between runs */
    uint64_t overflowed;     /* inserts that found all 32 probe buckets full; each was placed after its level's
                                inserts, by all warps at once, with a chain of at most 4 displacements */
    double evict_ms;         /* device time of those placement phases */
} gpx_result;

typedef struct gpx_model gpx_model;
typedef struct gpx_explorer gpx_explorer;

/* Scalar facts of a loaded model (the header lines GPUexplore.cu:1890-1953 print). */
typedef struct {
    uint32_t liveness, nr_procs, bits_act, proc_nrstates, bits_statevector;
    uint32_t nbits_offset, max_buf_ints, nr_trans;
    uint32_t state_bits;     /* firstbit_statevector[nr_procs] */
    uint32_t key_words;      /* ceil(state_bits / 32) */
    uint32_t firstbit[33];
    uint32_t bits_state[32];
} gpx_model_info;

/* Device facts the reference prints at start-up (GPUexplore.cu:2004-2010). */
typedef struct {
    uint64_t total_global_mem;
    int32_t shared_mem_per_block, shared_mem_per_sm, max_threads_per_block, max_grid_size, sm_count;
    char name[256];
} gpx_device_info;

/* Text of a status code; the reference prints these conditions and exits
 * (GPUexplore.cu:522-528, 1985, 2001, 2164-2166). */
const char *gpx_status_string(int status);
/* GPX_ABI_VERSION of the library (no reference counterpart). */
int gpx_abi_version(void);
/* GPX_ERR_NO_GPU when no CUDA device is present (GPUexplore.cu:1999-2003). */
int gpx_device_info_get(int device, gpx_device_info *info);

/* Defaults of the options (the reference's argv defaults, GPUexplore.cu:102-104, 1805-1883;
 * blocks/threads/levels per launch default to the whole GPU in one launch). */
void gpx_options_init(gpx_options *opts);

/* Load <path_without_ext>.gpf, appending the extension like GPUexplore.cu:1814-1815. */
int gpx_model_load(const char *path_without_ext, gpx_model **out);
/* Load a gpf file by its exact path (the reading of GPUexplore.cu:1885-1987). */
int gpx_model_load_file(const char *path, gpx_model **out);
/* Parse gpf integers already in host memory, one integer per gpf line (the same
 * reading without a file, GPUexplore.cu:1885-1987). */
int gpx_model_from_words(const uint32_t *words, size_t nwords, gpx_model **out);
int gpx_model_info_get(const gpx_model *model, gpx_model_info *info);
/* Release a model (no reference counterpart: the reference never releases its arrays). */
void gpx_model_free(gpx_model *model);

/* One-shot exploration: allocate, explore, free (the reference's main, GPUexplore.cu:1989-2172). */
int gpx_explore(const gpx_model *model, const gpx_options *opts, gpx_result *result);

/* Reusable explorer: the one-shot exploration split into allocation (create),
 * runs (the reset and exploration loop of GPUexplore.cu:2091-2142, each call) and
 * release (destroy).  Device memory (hash table, state store) is allocated once and
 * each run resets it, so repeated explorations pay no allocation. */
int gpx_explorer_create(const gpx_model *model, const gpx_options *opts, gpx_explorer **out);
int gpx_explorer_run(gpx_explorer *ex, gpx_result *result);
/* Replace the model of an explorer (host gpf integers, copied to the device by this
 * call); the new model must fit the explorer's key width. */
int gpx_explorer_set_model(gpx_explorer *ex, const gpx_model *model);
void gpx_explorer_destroy(gpx_explorer *ex);

/* Release the arrays of a result (no reference counterpart: the reference prints its
 * results, GPUexplore.cu:2144-2172). */
void gpx_result_free(gpx_result *result);

/* Failure-detection self-test (no reference counterpart): runs the bounded
 * device-side wait used by the persistent kernel's grid barrier on a flag that
 * nothing sets, with a limit of `timeout_ns` (at most 10 s).  Returns
 * GPX_ERR_TIMEOUT with the time waited when the wait gave up as designed; the
 * CUDA context stays usable. */
int gpx_selftest_bounded_wait(int device, uint64_t timeout_ns, uint64_t *waited_ns);

/* Random-access roofline probe (no reference counterpart; a measurement aid):
 * gathers random 32-byte sectors from a `bytes`-sized device buffer with the
 * same load the hash-table probes use, and reports the sustained rate in
 * gathers per second.  Allocates and frees the buffer itself. */
int gpx_random_gather_probe(int device, uint64_t bytes, double *gathers_per_s);

/* Insert roofline probe (no reference counterpart; a measurement aid): random
 * 32-byte buckets of a `bytes`-sized device buffer, each read and then updated
 * by a 128-bit CAS on its first slot -- the insert's access, one random sector
 * read and one dirty sector written back -- in accesses per second.  Allocates
 * and frees the buffer itself. */
int gpx_random_insert_probe(int device, uint64_t bytes, double *inserts_per_s);

/* Exploration that allocates no memory -- no counterpart in the reference.
 *
 * For callers that must not call cudaMalloc: code that runs while a framework's
 * caching allocator owns the device memory (an allocation outside it can fail
 * at the memory cap or fragment its pool), and latency-sensitive loops where
 * cudaMalloc/cudaFree would synchronise the device.  The hash table, state
 * store, level counts and control block live in one file-scope static device
 * array of GPX_NOALLOC_SCRATCH_BYTES (64 MiB), which every GPU that loads the
 * library holds until the process exits; this call uses no cudaMalloc, cudaFree
 * or other allocating routine, on the device or the host.
 *
 * Sizes: opts->q_words (table, 32-bit words) and opts->store_states may be 0
 * (split what is left of the array after the control block, 8 MiB of level
 * counts and the model) or explicit; a request that does not fit in the array
 * is rejected with GPX_ERR_INVALID and a message on stderr.
 * Inputs: the model (host handle; its words are copied into the array).
 * Outputs: `result` as gpx_explorer_run fills it, except that
 * result->level_counts points at the caller's `level_counts` array (the first
 * min(nlevels, level_capacity) entries are written; result->nlevels is the full
 * count), states_buf stays NULL, no -v output is printed, and explore_ms /
 * kernel_ms are host wall-clock times.  Do not pass this result to
 * gpx_result_free.  No pinned host memory is used either: after each launch
 * the control block (about 1 KB) is copied back into the call's own stack.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call before
 * any stream capture.  CUDA loads a library's kernels and reserves its static
 * arrays lazily, on first use in a context (CUDA_MODULE_LOADING=LAZY, the
 * default): if this call is the first use of libgpx on a device, the array is
 * reserved inside it, so a caller under a memory cap makes one call (or any
 * other libgpx call) on the device at set-up, while memory is still free.  The
 * address is cached per device ordinal for the life of the process; after a
 * cudaDeviceReset of that device it is stale and the library must not be used
 * there again.  The work runs on the calling thread's per-thread default stream
 * (cudaStreamPerThread: it does not wait for other blocking streams), and the
 * call returns when it has finished.  Every call on a device shares the one
 * array and leaves its contents behind (each call clears what it needs
 * cleared), so calls whose GPU work overlaps -- from two host threads, or on two
 * streams -- race. */
#define GPX_NOALLOC_SCRATCH_BYTES (64u << 20)
int gpx_explore_noalloc(const gpx_model *model, const gpx_options *opts, uint64_t *level_counts,
                        uint32_t level_capacity, gpx_result *result);

/* ---- Learned cluster proposal for POR (no reference counterpart).
 *
 * With gpx_options.por == 2 (and a model set), the cluster each state expands is
 * the valid cluster closure with the lowest score of a 2-layer MLP over
 * GPX_POR_FEATURES small-integer features of the closure (its size, local
 * targets and successors of its members, their synchronisation degree, members
 * whose proviso holds, the process count, rules led, and the members' (process,
 * local state) pairs hashed into 32 counts).  Layer 1: int8 weights times the
 * integer features, summed exactly, then fp32 (acc * s1 + b1), ReLU, rounded to
 * bf16; layer 2: int8 weights times the bf16 activations, fp32 FMA in order,
 * then (acc * s2 + b2).  The proposal is re-checked -- non-empty, closed under
 * the per-process clusters, some member's proviso holds -- and plain cample's
 * choice is used when the check fails, so the reduction stays sound. */
#define GPX_POR_FEATURES 40
#define GPX_POR_HIDDEN 64
typedef struct {
    int8_t w1[GPX_POR_HIDDEN][GPX_POR_FEATURES];
    float s1[GPX_POR_HIDDEN];
    float b1[GPX_POR_HIDDEN];
    int8_t w2[GPX_POR_HIDDEN];
    float s2, b2;
} gpx_por_model;

/* One logged candidate of a state expanded with POR and the cycle proviso: its
 * features, the successors its members generate, how many of them were not yet
 * visited (the outcome used as training label), and plain cample's choice. */
typedef struct {
    uint8_t x[GPX_POR_FEATURES];
    uint32_t succ;
    uint32_t new_succ;
    uint32_t state_tag;      /* hash of the source state: rows of one state share it */
    uint8_t popc;
    uint8_t cample_choice;   /* 1 if plain cample picks this closure */
    uint8_t pad[2];
} gpx_por_log_row;

/* Use `model` for por == 2 (NULL: plain cample).  The model is copied. */
int gpx_explorer_set_por_model(gpx_explorer *ex, const gpx_por_model *model);
/* Log up to `capacity` candidate rows of states whose hash is 0 mod sample_every
 * during the decide pass of later runs (por with the cycle proviso); 0 turns
 * logging off.  gpx_explorer_get_por_log copies the rows of the last run. */
int gpx_explorer_set_por_log(gpx_explorer *ex, uint64_t capacity, uint32_t sample_every);
int gpx_explorer_get_por_log(gpx_explorer *ex, gpx_por_log_row *rows, uint64_t capacity, uint64_t *nrows);

/* Training of the proposal MLP on the GPU with this library's forward and
 * backward kernels (fp32 master weights, int8 fake-quantised weights and bf16
 * activations in the forward pass, straight-through gradients, Adam, mean
 * squared error), exported as a gpx_por_model. */
typedef struct {
    uint32_t struct_size;
    int32_t device;
    uint32_t epochs;
    uint32_t batch;
    float lr;
    float weight_decay;
    uint64_t seed;
} gpx_train_options;
void gpx_train_options_init(gpx_train_options *o);
int gpx_por_train(const uint8_t *x, const float *y, uint64_t rows, const gpx_train_options *o,
                  gpx_por_model *out, float *final_loss);
/* One forward and backward pass over `rows` rows with the given fp32 weights
 * (w1 [H][F], b1 [H], w2 [H], b2), as the training kernels compute them:
 * mean-squared-error loss and its gradients (for checking them). */
int gpx_por_grad(int device, const float *w1, const float *b1, const float *w2, float b2, const uint8_t *x,
                 const float *y, uint32_t rows, float *gw1, float *gb1, float *gw2, float *gb2, float *loss);

/* ---- Batched exploration (no reference counterpart: the reference explores one
 * network per process).  Many networks of uneven size explored in one
 * persistent launch; each has its own hash-table and state-store partition,
 * sized from an admission estimate, and its own BFS levels, closed by whichever
 * warp finishes a level's last work claim (no grid-wide barrier).  An instance
 * that overflows its partition is re-admitted in a later launch with four times
 * the capacity.  Results per instance equal gpx_explore's on the same network. */
typedef struct {
    uint32_t struct_size;
    int32_t property;       /* gpx_property */
    int32_t por;            /* 0: none, 1: cluster POR, 2: cluster POR with the learned proposal, 3: ample, 4: stubborn */
    int32_t cycle_proviso;
    uint64_t max_states;    /* state budget (0 = none) */
    uint64_t capacity;      /* states admitted (table + store partition); 0 = estimate */
} gpx_batch_job;

typedef struct {
    int32_t status;         /* gpx_status of this instance */
    int32_t stopped;        /* gpx_stop */
    int32_t verdict;        /* violated gpx_property or GPX_PROP_NONE */
    uint32_t nlevels;
    uint64_t states;
    uint64_t set_hash;      /* order-independent hash of the visited set */
    uint64_t capacity;      /* states admitted in the launch that finished it */
    double completion_ms;   /* device time from that launch's start to the instance's last level */
    uint32_t admissions;    /* launches the instance needed */
    uint32_t slot_bytes;    /* its hash-slot width: 4, 8 or 16 bytes, the narrowest its state vector fits */
} gpx_batch_item;

typedef struct {
    uint32_t struct_size;
    int32_t device;
    int32_t blocks;         /* 0: every SM at full occupancy */
    int32_t threads;        /* per block; 0 = 256 */
    int32_t claim;          /* states per work claim (the frontier tile) at least; 0 = 8 (claims grow with
                               a level: a quarter of a fair share per warp, up to 4096) */
    int32_t kernel_iters;   /* work claims per warp per launch (0 = until every instance is done) */
    int32_t autotune;       /* choose claim, threads, load factor, then kernel_iters, then the slot policy on a
                               sample of the batch, then the claim size on the whole batch (at most 1,024
                               instances) first (the explicit values above are the starting point) */
    int32_t max_admissions; /* launches per instance before an overflow is final (0 = 3) */
    double load_factor;     /* table slots = admitted states / load_factor (0 = 0.5) */
    uint64_t seed;
    const gpx_por_model *por_model; /* for jobs with por == 2 (NULL: plain cample) */
    int32_t latency_sms;    /* SMs that serve the small phases of deep instances (latency-bound) first:
                               -1 (gpx_batch_options_init) = a tenth of the SMs, 0 = none */
    int32_t prune_commuting; /* 1 (gpx_batch_options_init): plain instances prune commuting moves
                                (gpx_options.prune_commuting); 0: every successor */
    int32_t narrow_slots;   /* 1: each instance gets the narrowest hash slot its state vector fits (32, 64 or
                               128 bits: two to four times the states per byte for small networks); 0
                               (gpx_batch_options_init): 128-bit slots for every instance (two per bucket, fewer
                               concurrent inserts per sector: faster on many small instances) */
} gpx_batch_options;

typedef struct {
    double device_ms;       /* device time of all batch launches, autotuning excluded */
    uint64_t states;        /* states of all instances */
    double p50_ms, p99_ms;  /* per-instance completion times (first launch) */
    uint32_t launches;
    int32_t claim, threads, blocks;
    double load_factor;
    double tune_ms;         /* host time spent autotuning */
    int32_t kernel_iters;   /* claims per warp per launch that ran (tuned with autotune) */
    uint32_t instances_by_slot[3]; /* instances with 32-, 64- and 128-bit slots */
    int32_t narrow_slots;   /* the slot policy that ran (tuned with autotune) */
} gpx_batch_stats;

void gpx_batch_options_init(gpx_batch_options *opts);
void gpx_batch_job_init(gpx_batch_job *job);
/* models[count], jobs[count], items[count]; level_counts (optional) receives
 * count x level_capacity per-level counts, row i for instance i. */
int gpx_batch_explore(const gpx_model *const *models, const gpx_batch_job *jobs, uint32_t count,
                      const gpx_batch_options *opts, gpx_batch_item *items, uint64_t *level_counts,
                      uint32_t level_capacity, gpx_batch_stats *stats);

/* Write the visited set of the last run in the reference's --dump format
 * (print_local_queue, GPUexplore.cu:594-612): one state per line, local states
 * comma separated, then the stripped state-vector words. */
int gpx_explorer_dump(gpx_explorer *ex, const char *path);

#ifdef __cplusplus
}
#endif

#endif /* GPX_H */
