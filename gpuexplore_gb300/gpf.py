"""The gpf network-of-LTSs format: an abstract network model, a writer and a reader.

A gpf file holds one unsigned integer per line, in the order the reference's
loader reads them (GPUexplore/src/GPUexplore.cu:1885-1987):

    liveness flag, nr_procs, bits_act, proc_nrstates, bits_statevector,
    firstbit_statevector[nr_procs+1], bits_state[nr_procs], nbits_offset,
    max_buf_ints, proc_offsets_start[nr_procs+1],
    proc_offsets[proc_offsets_start[nr_procs]], nr_trans, proc_trans[nr_trans],
    nbits_syncbits_offset, nr_syncbits_offsets, syncbits_offsets[...],
    nr_syncbits, syncbits[...]

Field packing (the same bit layout the reference decodes):

* A process p's local state occupies bits [firstbit[p], firstbit[p+1]) of the
  little-endian word array of a state vector (GPUexplore.cu:162-178).
* proc_offsets: process p's words start at proc_offsets_start[p]; local state
  s's transition range is fields s and s+1, each nbits_offset wide, packed
  32 // nbits_offset to a word from bit 0 (GPUexplore.cu:883-898).
* proc_trans entry: bit 0 = synchronising flag, bits [1, 1+bits_act) = action,
  then (31-bits_act) // bits_state[p] target slots of bits_state[p] bits each,
  holding target+1 (0 = unused) (GPUexplore.cu:143, 157-159).  Per (p, s) the
  local entries come first, then synchronising entries grouped by ascending
  action (required by the minimum-action merge at GPUexplore.cu:979-995).
  Targets are packed densely: an entry is only followed by another entry for
  the same action when all of its slots are used (the reference's successor
  odometer, GPUexplore.cu:1093-1108, stops at the first empty slot).
* syncbits_offsets: fields of nbits_syncbits_offset bits; action a's rules are
  the words [field a, field a+1) of syncbits (GPUexplore.cu:998-1009).
* syncbits: each word packs 32 // nr_procs rules of nr_procs bits; a rule is
  the bitmask of participating processes, 0 is padding (GPUexplore.cu:1018-1019,
  205).

The abstract :class:`Network` is what the generators build; :func:`encode`
turns it into gpf words and :func:`decode` turns gpf words back into a
:class:`Network`.  The safety property, when a model carries one, is embedded
the way the reference checks it: the last process is a monitor whose local
state 1 is the error state (GPUexplore.cu:927-935, 1063-1069).
"""
from __future__ import annotations

import random
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

MAX_PROCS = 31  # rule masks are (1 << nr_procs) - 1 wide (GPUexplore.cu:980, 995)


@dataclass
class Network:
    """A network of LTSs with synchronisation rules.

    nstates[p]      number of local states of process p (initial local state 0)
    local[p][s]     targets of p's local (non-synchronising) transitions from s
    sync[p][s]      {action: targets} of p's synchronising transitions from s
    rules[a]        list of participant bitmasks for synchronising action a
    liveness        the first gpf line (1 marks a liveness property)
    """

    nstates: List[int]
    local: List[List[List[int]]]
    sync: List[List[Dict[int, List[int]]]]
    rules: Dict[int, List[int]] = field(default_factory=dict)
    liveness: int = 0

    @property
    def nprocs(self) -> int:
        return len(self.nstates)

    def nactions(self) -> int:
        acts = set(self.rules)
        for p in range(self.nprocs):
            for s in range(self.nstates[p]):
                acts.update(self.sync[p][s])
        return (max(acts) + 1) if acts else 0

    def bits_state(self) -> List[int]:
        # slots hold target+1, so nstates must fit in the field (values 1..nstates)
        return [max(1, ns.bit_length()) for ns in self.nstates]

    def firstbit(self) -> List[int]:
        fb = [0]
        for b in self.bits_state():
            fb.append(fb[-1] + b)
        return fb

    def validate(self) -> None:
        n = self.nprocs
        if not 1 <= n <= MAX_PROCS:
            raise ValueError(f"nr_procs must be in 1..{MAX_PROCS}, got {n}")
        for p in range(n):
            if len(self.local[p]) != self.nstates[p] or len(self.sync[p]) != self.nstates[p]:
                raise ValueError(f"process {p}: transition lists do not match nstates")
            for s in range(self.nstates[p]):
                seen = set()
                for t in self.local[p][s]:
                    if not 0 <= t < self.nstates[p]:
                        raise ValueError(f"process {p} state {s}: local target {t} out of range")
                    if t in seen:
                        raise ValueError(f"process {p} state {s}: duplicate local target {t}")
                    seen.add(t)
                for a, ts in self.sync[p][s].items():
                    if not ts:
                        raise ValueError(f"process {p} state {s}: action {a} without targets")
                    if len(set(ts)) != len(ts):
                        raise ValueError(f"process {p} state {s}: duplicate targets for action {a}")
                    for t in ts:
                        if not 0 <= t < self.nstates[p]:
                            raise ValueError(f"process {p} state {s}: target {t} out of range")
        for a, rs in self.rules.items():
            for r in rs:
                if r <= 0 or r >> n:
                    raise ValueError(f"action {a}: rule mask {r:#x} invalid for {n} processes")


@dataclass
class GpfHeader:
    """Scalar header fields of a gpf file, as the reference's loader prints them."""

    liveness: int
    nr_procs: int
    bits_act: int
    proc_nrstates: int
    bits_statevector: int
    firstbit: List[int]
    bits_state: List[int]
    nbits_offset: int
    max_buf_ints: int
    nr_trans: int


def _pack_fields(values: Sequence[int], nbits: int) -> List[int]:
    per = 32 // nbits
    words = [0] * ((len(values) + per - 1) // per)
    for i, v in enumerate(values):
        if v >> nbits:
            raise ValueError(f"value {v} does not fit in {nbits} bits")
        words[i // per] |= v << ((i % per) * nbits)
    return words


def _field(words: Sequence[int], i: int, nbits: int) -> int:
    per = 32 // nbits
    return (words[i // per] >> ((i % per) * nbits)) & ((1 << nbits) - 1)


def encode(net: Network, max_slots: Optional[int] = None, repeat_seed: Optional[int] = None) -> List[int]:
    """Encode a network as the integer lines of a gpf file.

    By default every transition entry is packed densely and every target is
    written once, the form on which the reference's two successor kernels agree.
    Two options write the other forms the format allows (same Network, same
    successor sets under the intended semantics):

    max_slots    at most this many targets per entry; the remaining slots stay 0,
                 so one action's targets span more entries (max_buf_ints grows
                 past 2) and an entry with empty slots is followed by another
                 entry of the same action
    repeat_seed  seeded: about a third of the target lists get one of their
                 targets written a second time (the same successor twice)
    """
    net.validate()
    n = net.nprocs
    bs = net.bits_state()
    fb = net.firstbit()
    A = net.nactions()
    bits_act = max(1, (A - 1).bit_length()) if A > 0 else 1
    slots = [(31 - bits_act) // b for b in bs]
    if min(slots) < 1:
        raise ValueError("a process has too many local states for its transition entries")
    per_entry = [min(k, max_slots) if max_slots else k for k in slots]
    rng = random.Random(repeat_seed) if repeat_seed is not None else None

    def with_repeats(targets: List[int]) -> List[int]:
        if rng is None or rng.random() >= 1 / 3:
            return targets
        return targets + [rng.choice(targets)]

    trans: List[int] = []
    starts: List[List[int]] = []
    max_buf = 1
    for p in range(n):
        st = []
        for s in range(net.nstates[p]):
            st.append(len(trans))

            def entries(sync_flag: int, act: int, targets: List[int]) -> int:
                cnt = 0
                for c in range(0, len(targets), per_entry[p]):
                    e = sync_flag | (act << 1)
                    for i, t in enumerate(targets[c:c + per_entry[p]]):
                        e |= (t + 1) << (1 + bits_act + i * bs[p])
                    trans.append(e)
                    cnt += 1
                return cnt

            if net.local[p][s]:
                entries(0, 0, with_repeats(list(net.local[p][s])))
            for a in sorted(net.sync[p][s]):
                max_buf = max(max_buf, entries(1, a, with_repeats(list(net.sync[p][s][a]))))
        st.append(len(trans))
        starts.append(st)

    nr_trans = len(trans)
    nbits_offset = max(1, nr_trans.bit_length())
    if nbits_offset > 31:
        raise ValueError("too many transition entries")
    proc_offsets: List[int] = []
    proc_offsets_start = [0]
    for p in range(n):
        proc_offsets.extend(_pack_fields(starts[p], nbits_offset))
        proc_offsets_start.append(len(proc_offsets))

    syncbits: List[int] = []
    soffs = []
    per_rule = 32 // n
    for a in range(A):
        soffs.append(len(syncbits))
        rs = net.rules.get(a, [])
        words = [0] * ((len(rs) + per_rule - 1) // per_rule)
        for i, r in enumerate(rs):
            words[i // per_rule] |= r << ((i % per_rule) * n)
        syncbits.extend(words)
    soffs.append(len(syncbits))
    nbits_sync = max(1, len(syncbits).bit_length())
    syncbits_offsets = _pack_fields(soffs, nbits_sync)

    out = [int(net.liveness), n, bits_act, min(slots), fb[n] + 1]
    out += fb
    out += bs
    out += [nbits_offset, max_buf]
    out += proc_offsets_start
    out += proc_offsets
    out += [nr_trans] + trans
    out += [nbits_sync, len(syncbits_offsets)] + syncbits_offsets
    out += [len(syncbits)] + syncbits
    return out


def write(net: Network, path: str) -> None:
    """Write a network to `path` (the caller chooses the name, normally *.gpf)."""
    with open(path, "w") as f:
        f.write("\n".join(str(v) for v in encode(net)))
        f.write("\n")


def read_words(path: str) -> List[int]:
    """Read the integer lines of a gpf file (atoi semantics, as unsigned 32-bit)."""
    words = []
    with open(path) as f:
        for line in f:
            line = line.strip()
            if not line:
                continue
            num = ""
            for i, ch in enumerate(line):
                if ch.isdigit() or (i == 0 and ch in "+-"):
                    num += ch
                else:
                    break
            v = int(num) if num not in ("", "+", "-") else 0
            words.append(v & 0xFFFFFFFF)
    return words


def decode(words: Sequence[int]) -> Network:
    """Decode gpf words into a Network (inverse of :func:`encode` up to entry packing)."""
    it = iter(words)
    nxt = lambda: next(it)  # noqa: E731
    liveness = nxt()
    n = nxt()
    bits_act = nxt()
    nxt()  # proc_nrstates (printed by the reference, otherwise unused)
    nxt()  # bits_statevector
    fb = [nxt() for _ in range(n + 1)]
    bs = [nxt() for _ in range(n)]
    nbits_offset = nxt()
    nxt()  # max_buf_ints
    pos = [nxt() for _ in range(n + 1)]
    poffs = [nxt() for _ in range(pos[n])]
    nr_trans = nxt()
    trans = [nxt() for _ in range(nr_trans)]
    nbits_sync = nxt()
    nso = nxt()
    soffs = [nxt() for _ in range(nso)]
    nsb = nxt()
    sbits = [nxt() for _ in range(nsb)]
    if any(fb[p + 1] - fb[p] != bs[p] for p in range(n)):
        raise ValueError("firstbit_statevector and bits_state disagree")

    nstates = []
    local: List[List[List[int]]] = []
    sync: List[List[Dict[int, List[int]]]] = []
    per = 32 // nbits_offset
    for p in range(n):
        nfields = (pos[p + 1] - pos[p]) * per
        words_p = poffs[pos[p]:pos[p + 1]]
        f = [_field(words_p, i, nbits_offset) for i in range(nfields)]
        # the encoder writes nstates+1 nondecreasing fields; padding fields are 0
        k = 0
        while k + 1 < nfields and f[k + 1] >= f[k]:
            k += 1
        ns = k if (nfields and f[k] > 0) else 0
        nslots = (31 - bits_act) // bs[p]
        lp: List[List[int]] = []
        sp: List[Dict[int, List[int]]] = []
        for s in range(ns):
            lt: List[int] = []
            sd: Dict[int, List[int]] = {}
            for e in trans[f[s]:f[s + 1]]:
                ts = []
                for i in range(nslots):
                    v = (e >> (1 + bits_act + i * bs[p])) & ((1 << bs[p]) - 1)
                    if v == 0:
                        break
                    ts.append(v - 1)
                if e & 1:
                    sd.setdefault((e >> 1) & ((1 << bits_act) - 1), []).extend(ts)
                else:
                    lt.extend(ts)
            lp.append(lt)
            sp.append(sd)
        used = max([ns, 1] + [t + 1 for lt in lp for t in lt]
                   + [t + 1 for sd in sp for ts in sd.values() for t in ts])
        nstates.append(used)
        local.append(lp + [[] for _ in range(used - ns)])
        sync.append(sp + [{} for _ in range(used - ns)])

    rules: Dict[int, List[int]] = {}
    nper = 32 // n
    nact = (len(soffs) * (32 // nbits_sync)) - 1
    for a in range(nact):
        o1 = _field(soffs, a, nbits_sync)
        o2 = _field(soffs, a + 1, nbits_sync)
        rs = []
        for w in range(o1, max(o1, o2)):
            for i in range(nper):
                r = (sbits[w] >> (i * n)) & ((1 << n) - 1)
                if r:
                    rs.append(r)
        if rs:
            rules[a] = rs
    return Network(nstates=nstates, local=local, sync=sync, rules=rules, liveness=liveness)


def header(words: Sequence[int]) -> GpfHeader:
    """The scalar header of a gpf file."""
    n = words[1]
    fb = list(words[5:5 + n + 1])
    bs = list(words[6 + n:6 + 2 * n])
    i = 6 + 2 * n
    nbits_offset, max_buf = words[i], words[i + 1]
    pos = list(words[i + 2:i + 3 + n])
    j = i + 3 + n + pos[n]
    return GpfHeader(liveness=words[0], nr_procs=n, bits_act=words[2], proc_nrstates=words[3],
                     bits_statevector=words[4], firstbit=fb, bits_state=bs,
                     nbits_offset=nbits_offset, max_buf_ints=max_buf, nr_trans=words[j])
