"""The single-buffer schedule of pe_grad's pipelined grouped reverse pass (k_grad_reverse_group,
PIPE) on the CPU.  Each flight keeps one segment of rebuilt entries; while warp 0 differentiates
segment sg from its last step down, warp 1 rebuilds segment sg - 1 into slots warp 0 has already
read and warp 2 evaluates each rebuilt entry one iteration later.  The slot map, the entry warp 1
rebuilds at each iteration and the count of entries rebuilt so far restate the kernel's lambdas
(slot, rb_entry, rb_count); the test replays the schedule for every flight length against the
block's longest and checks that no slot is written while it holds an entry still to be read, that
warps 0, 1 and 2 never touch one slot in the same iteration, and that every entry is rebuilt, then
evaluated, then read exactly once, at checkpoint intervals from 1 to the largest the pass takes."""
import random


def _schedule(K, kg, kmax):
    sLg = kg // K
    Lg = kg - sLg * K + 1

    def slot(s, n):
        d = sLg - s
        if d == 0:
            return n
        m = n if d & 1 else K - 1 - n
        return Lg - 1 - m if m < Lg else m

    def seg_len(s):
        j0 = s * K
        return min(K, kg - j0 + 1) if kg >= j0 else 0

    def rb_entry(sg, j1, i):
        return i if kg < sg * K else i - (j1 - min(j1, kg)) - 1

    def rb_count(sg, j1, i):
        return 0 if i <= 0 else max(0, min(seg_len(sg - 1), rb_entry(sg, j1, i - 1) + 1))

    buf, read = {}, set()

    def write(s, n):
        sl = slot(s, n)
        assert 0 <= sl < K
        if sl in buf:
            assert buf[sl][:2] in read, ("slot overwritten before it was read", K, kg, kmax, s, n)
        buf[sl] = (s, n, "rebuilt")

    def evaluate(s, n):
        assert buf.get(slot(s, n)) == (s, n, "rebuilt"), ("evaluated before rebuilt", K, kg, kmax, s, n)
        buf[slot(s, n)] = (s, n, "evaluated")

    def consume(s, n):
        assert buf.get(slot(s, n)) == (s, n, "evaluated"), ("read before evaluated", K, kg, kmax, s, n)
        assert (s, n) not in read
        read.add((s, n))

    S = kmax // K
    for n in range(seg_len(S)):
        write(S, n)
    for n in range(seg_len(S)):
        evaluate(S, n)
    for sg in range(S, -1, -1):
        j0 = sg * K
        j1 = min(j0 + K - 1, kmax)
        length = j1 - j0 + 1
        for i in range(length):
            j = j1 - i
            touched = []
            if j <= kg:
                touched.append(slot(sg, j - j0))
            w = e = None
            if sg >= 1:
                nb = rb_entry(sg, j1, i)
                if 0 <= nb < seg_len(sg - 1):
                    w = nb
                    touched.append(slot(sg - 1, nb))
                if i >= 1:
                    nb = rb_entry(sg, j1, i - 1)
                    if 0 <= nb < seg_len(sg - 1):
                        e = nb
                        touched.append(slot(sg - 1, nb))
            assert len(set(touched)) == len(touched), ("two warps on one slot", K, kg, kmax, sg, i)
            if j <= kg:
                consume(sg, j - j0)
            if w is not None:
                write(sg - 1, w)
            if e is not None:
                evaluate(sg - 1, e)
        if sg >= 1:
            for n in range(rb_count(sg, j1, length), seg_len(sg - 1)):
                write(sg - 1, n)
            for n in range(rb_count(sg, j1, length - 1), seg_len(sg - 1)):
                evaluate(sg - 1, n)
    assert read == {(s, n) for s in range(sLg + 1) for n in range(seg_len(s))}


def test_grouped_pass_slot_schedule():
    for K in (1, 2, 3, 7):
        for kmax in range(4 * K + 3):
            for kg in range(kmax + 1):
                _schedule(K, kg, kmax)
    rng = random.Random(1)
    for K in (59, 60):  # every pair of last-segment lengths, 1-3 segments apart
        for kmax in (K - 1, 2 * K + 16, 3 * K - 1):
            for kg in range(0, kmax + 1, 3):
                _schedule(K, kg, kmax)
    for K in (7, 60):
        for _ in range(100):
            kmax = rng.randint(0, 7199)
            _schedule(K, rng.randint(0, kmax) if rng.random() < 0.8 else kmax, kmax)
