// gpx_model.h -- gpf loading and the decoded device layout of a network.
//
// The reference reads the gpf file field by field (GPUexplore.cu:1885-1987) and
// decodes the packed bit fields inside its kernels on every visit
// (GPUexplore.cu:883-898, 157-161, 998-1019).  Here the host decodes the network
// once into flat per-(process, local state) records that a kernel keeps in
// shared memory: local targets, synchronising (action, targets) groups, the
// rules each process leads, and the static POR cluster.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace gpx {

constexpr int kMaxProcs = 31;      // rule masks are nr_procs bits (GPUexplore.cu:980, 995)
constexpr int kMaxStateBits = 126; // widest state vector a 128-bit slot holds (63 + 63 bits)
constexpr int kHdrWords = 160;     // words of the device-layout header
constexpr int kRecWords = 8;       // words per (process, local state) record

// Raw gpf fields, named as in the reference.
struct Gpf {
    uint32_t liveness = 0, nr_procs = 0, bits_act = 0, proc_nrstates = 0, bits_statevector = 0;
    std::vector<uint32_t> firstbit, bits_state;
    uint32_t nbits_offset = 0, max_buf_ints = 0;
    std::vector<uint32_t> proc_offsets_start, proc_offsets;
    uint32_t nr_trans = 0;
    std::vector<uint32_t> proc_trans;
    uint32_t nbits_syncbits_offset = 0, nr_syncbits_offsets = 0;
    std::vector<uint32_t> syncbits_offsets;
    uint32_t nr_syncbits = 0;
    std::vector<uint32_t> syncbits;
};

// Header word indices of the device layout.
enum HdrIndex : int {
    H_NPROCS = 0,
    H_STATE_BITS = 1,
    H_FB = 2,          // firstbit[0..nprocs]           (33 words)
    H_BS = 35,         // bits_state[0..nprocs-1]       (32 words)
    H_PSBASE = 67,     // record index of (p, 0)        (33 words)
    H_OFF_RECS = 100,  // offsets (in words) of the arrays below
    H_OFF_LTGT = 101,
    H_OFF_SENT = 102,
    H_OFF_STGT = 103,
    H_OFF_RULES = 104,
    H_OFF_LRULE = 105,
    H_NRULES = 106,
    H_TOTAL_WORDS = 107,
    H_MAX_LRULES = 108, // most rules led by one (process, state)
    H_PDESC = 128,      // per process: firstbit | bits_state << 7 | record base << 12 (32 words)
};

// Record fields (kRecWords words per (p, s)).
enum RecIndex : int {
    R_LOFF = 0,  // first local target in ltgt
    R_LCNT = 1,  // number of local targets
    R_SOFF = 2,  // first synchronising group in sent (4 words each)
    R_SCNT = 3,  // number of synchronising groups (distinct actions)
    R_ROFF = 4,  // first entry in lrule
    R_RCNT = 5,  // rules this process leads (lowest member) for actions it has enabled
    R_CL0 = 6,   // static POR cluster: {p} and every rule containing p of an enabled action
    R_FLAGS = 7, // bit 0: some local target is local state 1
};

// Synchronising group (4 words): action, first target in stgt, target count,
// flags: bit 0 = some target is local state 1, bits 1.. = index of the action's
// first rule (an action's rules are consecutive in the rules array).
struct Decoded {
    uint32_t nprocs = 0;
    uint32_t state_bits = 0;
    uint32_t key_words = 1;  // ceil(state_bits / 32)
    std::vector<uint32_t> nstates;
    std::vector<uint32_t> words; // the device layout, header first
};

// Parse gpf integers (one per line).  Returns an empty string on success, else
// a one-line reason.
std::string parse_gpf_text(const std::string &text, Gpf *out);
std::string parse_gpf_words(const uint32_t *w, size_t n, Gpf *out);
// Validate and decode into the device layout.
std::string decode_gpf(const Gpf &g, Decoded *out);

} // namespace gpx

// The opaque model handle of the C ABI (include/gpx.h).
struct gpx_model {
    gpx::Gpf gpf;
    gpx::Decoded dec;
};
