// gpx_live.h -- accepting-cycle (liveness) check over an explored state space.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace gpx {

// Scratch of the check, owned by the caller and grown on demand.
struct LiveScratch {
    uint32_t *index = nullptr;            // per table slot: the store position of the state in it
    uint32_t *flag = nullptr;             // per state: bit 0 in the candidate set, bit 1 marked
    uint32_t *indeg = nullptr;            // per state: predecessors inside the set
    uint32_t *front[2] = {nullptr, nullptr}; // frontiers of store positions
    unsigned long long *count = nullptr;  // device counters
    unsigned long long slots = 0, states = 0;
    // the successor relation as edge lists: per state its out-degree and first edge
    uint32_t *deg = nullptr;
    unsigned long long *beg = nullptr;
    uint32_t *edges = nullptr;            // store positions of the successors
    unsigned long long lists_cap = 0, edges_cap = 0;
};

void live_free(LiveScratch *s);

// After a complete exploration: does a cycle of the full transition relation
// pass through a state whose last process is in local state 1?  `table` holds
// exactly the visited states and `store` lists them (positions 0..states-1;
// slot form by kind: 0 = 32, 1 = 64, 2 = 128 bits, 3 = 128 bits with a run
// generation, whose older-generation slots count as free); `model` is the decoded
// device layout.  On success *set_states is the size of the final candidate set
// (0: no accepting cycle) and *rounds the frontier rounds.
int live_check(int kind, void *table, unsigned long long nbuckets, unsigned long long slots, const void *store,
               unsigned long long states, const uint32_t *model, unsigned long long seed, cudaStream_t st,
               LiveScratch *s, unsigned long long *set_states, unsigned long long *rounds);

} // namespace gpx
