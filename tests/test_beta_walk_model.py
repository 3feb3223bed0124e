"""CPU model of the beta kernel's walk formulations against the plain automaton.

BetaGen's general branch (EigenRand/Dists/NormalExp.h:970-975) draws one
packet from GammaGen(a), then one from GammaGen(b); a GS component
(NormalExp.h:527-553) runs trials of three packets through CompressMask
(arch/AVX/PacketFilter.h:147-184): a fully accepted trial is the output
packet and leaves the carried lanes alone; otherwise the accepted lanes are
appended to the carry, and once it holds P lanes its oldest P are the output.

k_beta resolves that automaton from accept masks evaluated ahead of the walk.
On engines that share an SM the chase walks trial by trial and writes the
FIFO slots itself.  For single-engine calls it reads a visit table: per
position x and carry f, where the GS visit starting there ends, whether on a
full trial, and how many lanes its partial trials accept; the chase reads one
entry per output packet and records the visit's start, carry and FIFO tail,
and the workers walk each visit again one step later to place its accepted
lanes.  The kernel keeps
masks and table entries in 1024-slot rings, evaluates masks one engine block
(312 packets) at a time, leaves an entry unknown while its visit runs past the
evaluated masks, rebuilds unknown entries with the next block's masks (the
chase may read an entry while it is rebuilt), and never looks further back
than two blocks.  This model follows those steps and checks every output
packet's sources, the FIFO lane order, the final position and carry against a
direct restatement of the automaton, on random masks, for both forms.
"""
import random

import pytest

KN, RING = 312, 1024
NONE = None


def popc(m):
    return bin(m).count("1")


def automaton(mask_at, P, ug, uc, order, f0, npk):
    """The reference's draw loop: GS visits and closed-form draws in order."""
    x, f, A = 0, f0, f0
    recs, fifo = [], []
    for _ in range(npk):
        rec = []
        for c in order:
            if c == "closed":
                rec.append(("pos", x))
                x += uc
                continue
            while True:
                m = mask_at(x)
                cn = popc(m)
                if cn == P:
                    rec.append(("full", x))
                    x += ug
                    break
                fifo += [(x, j) for j in range(P) if m >> j & 1]
                A += cn
                f += cn
                x += ug
                if f >= P:
                    rec.append(("fifo", A - f))
                    f -= P
                    break
        recs.append(tuple(rec))
    return recs, fifo, x, f


def table_pipeline(mask_at, P, ug, uc, order, f0, npk, rng, rec_cap=160, fifo_cap=112):
    """The single-engine k_beta steps: masks per block, visit table, chase one
    step ahead of the expansion, rings of RING slots."""
    lb = 16 + fifo_cap * P
    umax = max(ug, uc, 3)
    pmask = [0] * RING
    vtab = [[NONE] * P for _ in range(RING)]

    def M_of(t):
        return (t + 1) * KN - umax + 1

    def write_masks(a, b):
        for x in range(a, b):
            pmask[x % RING] = mask_at(x)

    def build(a, b, to):
        inv = None
        for x in range(a, b):
            for f in range(P):
                e, acc = NONE, 0
                for d in range(0, 1024 - ug, ug):
                    xr = x + d
                    if xr >= to:
                        break
                    m = pmask[xr % RING]
                    cn = popc(m)
                    if cn == P:
                        e = (d, True, acc)
                        break
                    acc += cn
                    if f + acc >= P:
                        e = (d, False, acc)
                        break
                vtab[x % RING][f] = e
                if e is NONE:
                    inv = x if inv is None else min(inv, x)
        return inv

    write_masks(0, M_of(0))
    inv = build(0, M_of(0), M_of(0))
    first_unknown = inv if inv is not None else M_of(0)
    cx, cf, ce, done = 0, f0, 0, False
    steps, out, carry = {}, [], [("carried", i) for i in range(f0)]
    t = 0
    while True:
        M, pk_lim = M_of(t), (t + 1) * KN
        if not done:
            view = [row[:] for row in vtab]
            if t % 2:  # entries rebuilt in this iteration, seen by the chase at random
                saved_m, saved_t = pmask[:], [row[:] for row in vtab]
                write_masks(M, M + KN)
                build(max(min(first_unknown, M), (t - 1) * KN), M + KN, M + KN)
                for x in range(max(0, (t - 1) * KN), M):
                    if rng.random() < 0.5:
                        view[x % RING] = vtab[x % RING][:]
                pmask[:] = saved_m
                vtab[:] = saved_t
            assert cx >= (t - 1) * KN, "the chase fell more than two blocks behind"
            base, fs, A, recs, starts = cx, cf, cf, [], []
            while ce < npk and len(recs) < rec_cap:
                saved = (cx, cf, A)
                rec, start, ok = [], None, True
                for c in order:
                    if c == "closed":
                        if cx + uc > pk_lim:
                            ok = False
                            break
                        rec.append(("pos", cx))
                        cx += uc
                        continue
                    e = view[cx % RING][cf] if cx < M else NONE
                    if e is NONE or A + e[2] > lb:
                        ok = False
                        break
                    d, full, acc = e
                    start = (cx, A, cf)
                    rec.append(("full", cx + d) if full else ("fifo", A - cf))
                    cf += acc if full else acc - P
                    A += acc
                    cx += d + ug
                if not ok:
                    cx, cf, A = saved
                    break
                recs.append(tuple(rec))
                starts.append(start)
                ce += 1
            steps[t] = (fs, A, cf, recs, starts)
            finished = ce >= npk
        # workers: step t - 1, before this iteration's masks overwrite ring slots
        if t >= 1 and steps.get(t - 1) and steps[t - 1][3]:
            fs, a_end, f_end, recs, starts = steps[t - 1]
            slots = {}
            for xs, a0, fv in starts:
                run, xr = 0, xs
                while True:
                    m = pmask[xr % RING]
                    assert m == mask_at(xr), "a mask slot was overwritten before its last use"
                    cn = popc(m)
                    if cn == P:
                        break
                    for j in range(P):
                        if m >> j & 1:
                            slots[a0 - fs + run + popc(m & ((1 << j) - 1))] = (xr, j)
                    run += cn
                    if fv + run >= P:
                        break
                    xr += ug
            lanes = carry + [slots[i] for i in range(a_end - fs)]
            for rec in recs:
                out.append(tuple(("fifo", tuple(lanes[i[1]:i[1] + P])) if i[0] == "fifo" else i for i in rec))
            carry = lanes[a_end - f_end:a_end]
        if done:
            break
        write_masks(M, M + KN)
        inv = build(max(min(first_unknown, M), (t - 1) * KN), M + KN, M + KN)
        first_unknown = inv if inv is not None else M + KN
        done = finished
        t += 1
    return out, carry, cx, cf


def trial_pipeline(mask_at, P, ug, uc, order, f0, npk, rec_cap=160, fifo_cap=112):
    """The k_beta steps on engines that share an SM: the chase walks trial by
    trial over the masks (positions below the evaluated limit only) and writes
    each accepted partial lane's FIFO slot itself; a record that does not fit
    rolls back to the next step; the workers read the slots one step later."""
    lb = 16 + fifo_cap * P
    umax = max(ug, uc, 3)
    pmask = [0] * RING

    def M_of(t):
        return (t + 1) * KN - umax + 1

    for x in range(M_of(0)):
        pmask[x % RING] = mask_at(x)
    cx, cf, ce, done = 0, f0, 0, False
    steps, out, carry = {}, [], [("carried", i) for i in range(f0)]
    t = 0
    while True:
        M, pk_lim = M_of(t), (t + 1) * KN
        if not done:
            assert cx >= (t - 1) * KN, "the chase fell more than two blocks behind"
            base, fs, A, recs, slots = cx, cf, cf, [], {}
            while ce < npk and len(recs) < rec_cap:
                saved = (cx, cf, A, dict(slots))
                rec, ok = [], True
                for c in order:
                    if c == "closed":
                        if cx + uc > pk_lim:
                            ok = False
                            break
                        rec.append(("pos", cx))
                        cx += uc
                        continue
                    acc, xr, end = 0, cx, None
                    while end is None:
                        if xr >= M:
                            break
                        m = pmask[xr % RING]
                        cn = popc(m)
                        if cn == P:
                            end = ("full", xr)
                            cf += acc
                            break
                        if A + acc + cn > lb:
                            break
                        for j in range(P):
                            if m >> j & 1:
                                slots[A + acc - fs + popc(m & ((1 << j) - 1))] = (xr, j)
                        acc += cn
                        if cf + acc >= P:
                            end = ("fifo", A - cf)
                            cf += acc - P
                            break
                        xr += ug
                    if end is None:
                        ok = False
                        break
                    rec.append(end)
                    A += acc
                    cx = xr + ug
                if not ok:
                    cx, cf, A, slots = saved
                    break
                recs.append(tuple(rec))
                ce += 1
            steps[t] = (fs, A, cf, recs, slots)
            finished = ce >= npk
        if t >= 1 and steps.get(t - 1) and steps[t - 1][3]:
            fs, a_end, f_end, recs, slots = steps[t - 1]
            lanes = carry + [slots[i] for i in range(a_end - fs)]
            for rec in recs:
                out.append(tuple(("fifo", tuple(lanes[i[1]:i[1] + P])) if i[0] == "fifo" else i for i in rec))
            carry = lanes[a_end - f_end:a_end]
        if done:
            break
        for x in range(M, M + KN):
            pmask[x % RING] = mask_at(x)
        done = finished
        t += 1
    return out, carry, cx, cf


def _case(seed):
    rng = random.Random(seed)
    P = rng.choice([4, 8])  # double and float packets
    uc = rng.choice([2, 3, 7, 19])  # integral alpha of the closed-form component
    order = rng.choice([("gs", "closed"), ("closed", "gs")])  # beta(a < 1, b) and beta(a, b < 1)
    p = rng.choice([0.35, 0.5, 0.8, 0.95])  # lane acceptance
    f0 = rng.randrange(P)  # lanes carried from the last call
    npk = rng.choice([1, 7, 120, 900])
    cache = {}

    def mask_at(x):
        if x not in cache:
            cache[x] = sum((rng.random() < p) << j for j in range(P))
        return cache[x]

    ref, fifo, rx, rf = automaton(mask_at, P, 3, uc, order, f0, npk)
    lanes = [("carried", i) for i in range(f0)] + fifo
    want = [tuple(("fifo", tuple(lanes[i[1]:i[1] + P])) if i[0] == "fifo" else i for i in rec) for rec in ref]
    return mask_at, P, uc, order, f0, npk, want, (rx, rf)


@pytest.mark.parametrize("seed", range(12))
def test_trial_chase_pipeline_equals_automaton(seed):
    mask_at, P, uc, order, f0, npk, want, end = _case(seed)
    got, _, gx, gf = trial_pipeline(mask_at, P, 3, uc, order, f0, npk)
    assert got == want
    assert (gx, gf) == end


@pytest.mark.parametrize("seed", range(12))
def test_visit_table_pipeline_equals_automaton(seed):
    mask_at, P, uc, order, f0, npk, want, end = _case(seed)
    got, _, gx, gf = table_pipeline(mask_at, P, 3, uc, order, f0, npk, random.Random(seed + 100))
    assert got == want
    assert (gx, gf) == end
