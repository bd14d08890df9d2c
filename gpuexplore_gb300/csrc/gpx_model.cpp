// gpx_model.cpp -- gpf parsing (GPUexplore.cu:1885-1987) and decoding into the
// flat device layout described in gpx_model.h.
#include "gpx_model.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>

namespace gpx {

namespace {

struct Cursor {
    const uint32_t *w;
    size_t n, i = 0;
    bool ok = true;
    uint32_t next() {
        if (i >= n) {
            ok = false;
            return 0;
        }
        return w[i++];
    }
    std::vector<uint32_t> take(uint64_t count) {
        std::vector<uint32_t> v;
        if (count > n - std::min(n, i)) {
            ok = false;
            return v;
        }
        v.assign(w + i, w + i + count);
        i += count;
        return v;
    }
};

uint32_t packed_field(const uint32_t *words, uint32_t i, uint32_t nbits) {
    uint32_t per = 32 / nbits;
    return (words[i / per] >> ((i % per) * nbits)) & ((1u << nbits) - 1u);
}

} // namespace

std::string parse_gpf_words(const uint32_t *w, size_t n, Gpf *g) {
    Cursor c{w, n};
    *g = Gpf();
    // field order of GPUexplore.cu:1888-1982
    g->liveness = c.next();
    g->nr_procs = c.next();
    g->bits_act = c.next();
    g->proc_nrstates = c.next();
    g->bits_statevector = c.next();
    if (!c.ok) return "truncated header";
    if (g->nr_procs < 1 || g->nr_procs > (uint32_t)kMaxProcs) return "nr_procs outside 1..31";
    g->firstbit = c.take(g->nr_procs + 1);
    g->bits_state = c.take(g->nr_procs);
    g->nbits_offset = c.next();
    g->max_buf_ints = c.next();
    g->proc_offsets_start = c.take(g->nr_procs + 1);
    if (!c.ok) return "truncated process layout";
    g->proc_offsets = c.take(g->proc_offsets_start[g->nr_procs]);
    g->nr_trans = c.next();
    if (!c.ok) return "truncated offsets";
    g->proc_trans = c.take(g->nr_trans);
    g->nbits_syncbits_offset = c.next();
    g->nr_syncbits_offsets = c.next();
    if (!c.ok) return "truncated transitions";
    g->syncbits_offsets = c.take(g->nr_syncbits_offsets);
    g->nr_syncbits = c.next();
    if (!c.ok) return "truncated synchronisation offsets";
    g->syncbits = c.take(g->nr_syncbits);
    if (!c.ok) return "truncated synchronisation rules";
    return "";
}

std::string parse_gpf_text(const std::string &text, Gpf *g) {
    // one integer per line with atoi semantics; values are kept as 32-bit words
    std::vector<uint32_t> words;
    size_t pos = 0;
    while (pos < text.size()) {
        size_t end = text.find('\n', pos);
        if (end == std::string::npos) end = text.size();
        std::string line = text.substr(pos, end - pos);
        pos = end + 1;
        size_t k = 0;
        while (k < line.size() && (line[k] == ' ' || line[k] == '\t' || line[k] == '\r')) k++;
        if (k == line.size()) continue;
        words.push_back((uint32_t)std::strtoll(line.c_str() + k, nullptr, 10));
    }
    return parse_gpf_words(words.data(), words.size(), g);
}

std::string decode_gpf(const Gpf &g, Decoded *out) {
    const uint32_t n = g.nr_procs;
    if (g.bits_act < 1 || g.bits_act > 30) return "bits_act outside 1..30";
    if (g.nbits_offset < 1 || g.nbits_offset > 31) return "nbits_offset outside 1..31";
    if (g.nbits_syncbits_offset < 1 || g.nbits_syncbits_offset > 31) return "nbits_syncbits_offset outside 1..31";
    if (g.firstbit[0] != 0) return "firstbit_statevector[0] != 0";
    for (uint32_t p = 0; p < n; p++) {
        if (g.bits_state[p] < 1 || g.bits_state[p] > 31 - g.bits_act) return "bits_state outside 1..31-bits_act";
        if (g.firstbit[p + 1] != g.firstbit[p] + g.bits_state[p]) return "firstbit_statevector disagrees with bits_state";
        if (g.proc_offsets_start[p + 1] < g.proc_offsets_start[p]) return "proc_offsets_start decreasing";
    }
    const uint32_t state_bits = g.firstbit[n];
    const uint32_t per_off = 32 / g.nbits_offset;

    // rules per action (GPUexplore.cu:998-1019): words [field a, field a+1) of syncbits
    const uint32_t per_sync_off = 32 / g.nbits_syncbits_offset;
    const uint64_t nact_fields = (uint64_t)g.nr_syncbits_offsets * per_sync_off;
    auto rules_of = [&](uint32_t a, std::vector<uint32_t> *masks) -> std::string {
        masks->clear();
        if ((uint64_t)a + 1 >= nact_fields) return "";
        uint32_t o1 = packed_field(g.syncbits_offsets.data(), a, g.nbits_syncbits_offset);
        uint32_t o2 = packed_field(g.syncbits_offsets.data(), a + 1, g.nbits_syncbits_offset);
        const uint32_t per_rule = 32 / n;
        for (uint32_t w = o1; w < o2; w++) {
            if (w >= g.nr_syncbits) return "synchronisation rule range past syncbits";
            for (uint32_t f = 0; f < per_rule; f++) {
                uint32_t r = (g.syncbits[w] >> (f * n)) & ((n == 32) ? 0xFFFFFFFFu : ((1u << n) - 1u));
                if (r) masks->push_back(r);
            }
        }
        return "";
    };

    // Decode every (p, s) reachable in p's LTS from local state 0 into flat
    // arrays: per state, its local targets (entry order, each once) and its
    // synchronising (action, target) pairs (ascending action, entry order within
    // an action, each pair once).  Ranges into the arrays per state; no
    // allocation per state.
    struct StateTr {
        uint32_t lb, le, sb, se; // [lb, le) of loc, [sb, se) of sy
    };
    std::vector<std::vector<StateTr>> tr(n);
    std::vector<uint32_t> loc;
    std::vector<uint64_t> sy; // action << 32 | target
    std::vector<uint32_t> nstates(n);
    std::vector<uint32_t> todo;
    std::vector<char> seen;
    for (uint32_t p = 0; p < n; p++) {
        const uint32_t nwords = g.proc_offsets_start[p + 1] - g.proc_offsets_start[p];
        const uint32_t nfields = nwords * per_off;
        const uint32_t *base = g.proc_offsets.data() + g.proc_offsets_start[p];
        const uint32_t w = g.bits_state[p], nslots = (31 - g.bits_act) / w;
        // every reachable local state s needs offset fields s and s+1, so state
        // indices are bounded by the input, whatever bits_state allows
        if (nfields < 2) return "transition offsets missing for a reachable local state";
        seen.assign(nfields, 0);
        std::vector<StateTr> &trp = tr[p];
        trp.assign(nfields, StateTr{0, 0, 0, 0});
        todo.assign(1, 0);
        seen[0] = 1;
        uint32_t maxs = 0;
        while (!todo.empty()) {
            uint32_t s = todo.back();
            todo.pop_back();
            maxs = std::max(maxs, s);
            if (s + 1 >= nfields) return "transition offsets missing for a reachable local state";
            uint32_t o1 = packed_field(base, s, g.nbits_offset);   // GPUexplore.cu:883-898
            uint32_t o2 = packed_field(base, s + 1, g.nbits_offset);
            StateTr &t0 = trp[s];
            t0.lb = (uint32_t)loc.size();
            t0.sb = (uint32_t)sy.size();
            for (uint32_t k = o1; k < o2; k++) {
                if (k >= g.nr_trans) return "transition range past proc_trans";
                uint32_t e = g.proc_trans[k];
                uint32_t nts = 0;
                const uint64_t act = (uint64_t)((e >> 1) & ((1u << g.bits_act) - 1u)) << 32;
                for (uint32_t i = 0; i < nslots; i++) {  // slots hold target+1 (GPUexplore.cu:159)
                    uint32_t t = (e >> (1 + g.bits_act + i * w)) & ((1u << w) - 1u);
                    if (!t) break;
                    t -= 1;
                    nts++;
                    if (e & 1u) {
                        const uint64_t at = act | t;
                        if (std::find(sy.begin() + t0.sb, sy.end(), at) == sy.end()) sy.push_back(at);
                    } else if (std::find(loc.begin() + t0.lb, loc.end(), t) == loc.end()) {
                        loc.push_back(t);
                    }
                    if (t + 1 >= nfields) return "transition offsets missing for a reachable local state";
                    if (!seen[t]) {
                        seen[t] = 1;
                        todo.push_back(t);
                    }
                }
                if (!nts) return "transition entry without targets";
            }
            t0.le = (uint32_t)loc.size();
            t0.se = (uint32_t)sy.size();
            // group by action, keeping entry order within an action
            std::stable_sort(sy.begin() + t0.sb, sy.end(),
                             [](uint64_t x, uint64_t y) { return (x >> 32) < (y >> 32); });
        }
        nstates[p] = maxs + 1;
        trp.resize(nstates[p]);
        for (uint32_t st = 0; st <= maxs; st++)
            if (!seen[st]) trp[st] = StateTr{0, 0, 0, 0};
    }
    if (state_bits > (uint32_t)kMaxStateBits) return "UNSUPPORTED: state vector wider than 126 bits";

    // rules, and per (p, s) the rules p leads (lowest member) for actions p has enabled
    std::vector<uint32_t> rule_mask, rule_act;
    std::vector<uint32_t> actions; // ascending, each once
    actions.reserve(sy.size());
    for (uint64_t at : sy) actions.push_back((uint32_t)(at >> 32));
    std::sort(actions.begin(), actions.end());
    actions.erase(std::unique(actions.begin(), actions.end()), actions.end());
    std::vector<std::pair<uint32_t, uint32_t>> ranges(actions.size()); // per action: [first rule, count)
    auto rules_range = [&](uint32_t a) -> const std::pair<uint32_t, uint32_t> & {
        return ranges[std::lower_bound(actions.begin(), actions.end(), a) - actions.begin()];
    };
    std::vector<uint32_t> masks;
    for (size_t i = 0; i < actions.size(); i++) {
        std::string err = rules_of(actions[i], &masks);
        if (!err.empty()) return err;
        ranges[i] = {(uint32_t)rule_mask.size(), (uint32_t)masks.size()};
        for (uint32_t m : masks) {
            rule_mask.push_back(m);
            rule_act.push_back(actions[i]);
        }
    }

    std::vector<uint32_t> recs, ltgt, sent, stgt, lrule;
    std::vector<uint32_t> psbase(n + 1, 0);
    uint32_t max_lrules = 0;
    for (uint32_t p = 0; p < n; p++) {
        psbase[p] = (uint32_t)(recs.size() / kRecWords);
        for (uint32_t s = 0; s < nstates[p]; s++) {
            const StateTr &r = tr[p][s];
            uint32_t rec[kRecWords] = {0};
            rec[R_LOFF] = (uint32_t)ltgt.size();
            rec[R_LCNT] = r.le - r.lb;
            for (uint32_t k = r.lb; k < r.le; k++) {
                ltgt.push_back(loc[k]);
                if (loc[k] == 1) rec[R_FLAGS] |= 1u;
            }
            rec[R_SOFF] = (uint32_t)(sent.size() / 4);
            rec[R_ROFF] = (uint32_t)lrule.size();
            uint32_t cl0 = 1u << p, groups = 0;
            for (uint32_t k = r.sb; k < r.se;) {  // one group per action, ascending
                const uint32_t a = (uint32_t)(sy[k] >> 32);
                uint32_t has1 = 0;
                const uint32_t toff = (uint32_t)stgt.size();
                for (; k < r.se && (uint32_t)(sy[k] >> 32) == a; k++) {
                    const uint32_t t = (uint32_t)sy[k];
                    stgt.push_back(t);
                    if (t == 1) has1 = 1;
                }
                const auto &rr = rules_range(a);
                sent.push_back(a);
                sent.push_back(toff);
                sent.push_back((uint32_t)stgt.size() - toff);
                sent.push_back(has1 | (rr.first << 1)); // + first rule of the action
                for (uint32_t q = rr.first; q < rr.first + rr.second; q++) {
                    uint32_t m = rule_mask[q];
                    if (m >> p & 1u) cl0 |= m; // GPUexplore.cu:1616-1624
                    if ((uint32_t)__builtin_ctz(m) == p) lrule.push_back(q);
                }
                groups++;
            }
            rec[R_SCNT] = groups;
            rec[R_RCNT] = (uint32_t)lrule.size() - rec[R_ROFF];
            rec[R_CL0] = cl0;
            max_lrules = std::max(max_lrules, rec[R_RCNT]);
            recs.insert(recs.end(), rec, rec + kRecWords);
        }
    }
    psbase[n] = (uint32_t)(recs.size() / kRecWords);
    if (max_lrules > 32) return "UNSUPPORTED: a process leads more than 32 rules in one local state";
    if (psbase[n] >= (1u << 20)) return "UNSUPPORTED: more than 2^20 (process, local state) records";

    std::vector<uint32_t> &wds = out->words;
    wds.assign(kHdrWords, 0);
    wds[H_NPROCS] = n;
    wds[H_STATE_BITS] = state_bits;
    for (uint32_t p = 0; p <= n; p++) wds[H_FB + p] = g.firstbit[p];
    for (uint32_t p = 0; p < n; p++) wds[H_BS + p] = g.bits_state[p];
    for (uint32_t p = 0; p <= n; p++) wds[H_PSBASE + p] = psbase[p];
    for (uint32_t p = 0; p < n; p++) wds[H_PDESC + p] = g.firstbit[p] | (g.bits_state[p] << 7) | (psbase[p] << 12);
    auto append = [&](const std::vector<uint32_t> &v) {
        uint32_t off = (uint32_t)wds.size();
        wds.insert(wds.end(), v.begin(), v.end());
        while (wds.size() % 4) wds.push_back(0); // keep every array 16-byte aligned
        return off;
    };
    wds[H_OFF_RECS] = append(recs);
    wds[H_OFF_LTGT] = append(ltgt);
    wds[H_OFF_SENT] = append(sent);
    wds[H_OFF_STGT] = append(stgt);
    std::vector<uint32_t> rules;
    for (size_t k = 0; k < rule_mask.size(); k++) {
        rules.push_back(rule_mask[k]);
        rules.push_back(rule_act[k]);
    }
    wds[H_OFF_RULES] = append(rules);
    wds[H_OFF_LRULE] = append(lrule);
    wds[H_NRULES] = (uint32_t)rule_mask.size();
    wds[H_TOTAL_WORDS] = (uint32_t)wds.size();
    wds[H_MAX_LRULES] = max_lrules;
    out->nprocs = n;
    out->state_bits = state_bits;
    out->key_words = state_bits ? (state_bits + 31) / 32 : 1;
    out->nstates = nstates;
    return "";
}

} // namespace gpx
