"""The insertion protocol of generation-tagged 128-bit slots, checked over every
interleaving of two inserting threads.

A model of find_or_insert on a probe sequence of two slots.  A bucket read
returns the two 64-bit halves of a slot as two separate atomic reads, in either
order, so a read can see one half before and one after another thread's CAS.
The slot itself changes only by a full-slot CAS.  A half belongs to the current
run when its generation tag matches.  Free = neither half current; torn =
exactly one half current (re-read atomically); otherwise the slot holds a key
of this run.  With the tag in both halves every key ends up in the table
exactly once.  With the tag in the high half only, a read of (stale low half,
new high half) can equal a different key, which is then reported as present
and lost.
"""
import itertools

GEN = 2  # the current run's generation; slots hold keys of generation 1


def _key(lo, hi, both=True):
    return ((GEN if both else None, lo), (GEN, hi))


def _stale(lo, hi, both=True):
    return ((1 if both else None, lo), (1, hi))


def _thread(slots, key, both, order):
    """Generator: one atomic step per yield; returns "inserted" or "found"."""
    def cur(half):
        return half[0] == GEN

    for j in range(len(slots)):
        first, second = order[j]
        obs = [None, None]
        obs[first] = slots[j][first]
        yield
        obs[second] = slots[j][second]
        yield
        v = tuple(obs)
        if both:
            free = not cur(v[0]) and not cur(v[1])
            torn = cur(v[0]) != cur(v[1])
        else:  # only the high half carries the tag: the low half's age is unknown
            free = not cur(v[1])
            torn = False
        if torn:
            v = slots[j]  # atomic re-read of the whole slot
            yield
            free = not cur(v[0]) and not cur(v[1])
        if v == key:
            return "found"
        if free:
            old = slots[j]  # full-slot CAS against what was read
            if old == v:
                slots[j] = key
            yield
            if old == v:
                return "inserted"
            if old == key:
                return "found"
    return "full"


def _explore(initial, keys, both):
    """Every schedule of the threads and every half-read order; yields
    (final slots, results)."""
    orders = list(itertools.product([(0, 1), (1, 0)], repeat=len(initial)))
    for per_thread in itertools.product(orders, repeat=len(keys)):
        # depth-first over schedules: replay a schedule prefix each time
        prefixes = [()]
        while prefixes:
            prefix = prefixes.pop()
            slots = list(initial)
            gens = [_thread(slots, k, both, per_thread[i]) for i, k in enumerate(keys)]
            results = [None] * len(keys)
            alive = set(range(len(keys)))

            def step(t):
                try:
                    next(gens[t])
                except StopIteration as e:
                    results[t] = e.value
                    alive.discard(t)

            for t in prefix:
                step(t)
            if not alive:
                yield slots, results
                continue
            for t in sorted(alive):
                prefixes.append(prefix + (t,))


def _check(initial, keys, both):
    bad = []
    for slots, results in _explore(initial, keys, both):
        for k, r in zip(keys, results):
            if slots.count(k) != 1 or r == "full":
                bad.append((slots, results))
        if len(set(keys)) == len(keys) and results.count("inserted") != len(keys):
            bad.append((slots, results))
        if len(set(keys)) == 1 and results.count("inserted") != 1:
            bad.append((slots, results))
    return bad


def test_two_threads_one_key_exactly_once():
    """Two threads insert the same key over stale contents: one inserts, one finds."""
    k = _key(5, 9)
    assert not _check([_stale(5, 9), _stale(3, 4)], [k, k], both=True)


def test_false_match_needs_the_tag_in_both_halves():
    """X is inserted over a stale slot whose low half equals Y's, and Y shares
    X's high half: with both halves tagged every interleaving keeps both keys."""
    x, y = _key(7, 9), _key(5, 9)
    assert not _check([_stale(5, 3), _stale(0, 0)], [x, y], both=True)
    x1, y1 = _key(7, 9, both=False), _key(5, 9, both=False)
    bad = _check([_stale(5, 3, both=False), _stale(0, 0, both=False)], [x1, y1], both=False)
    assert bad  # some interleaving reports Y present when it is not
    assert any(y1 not in slots for slots, _ in bad)
