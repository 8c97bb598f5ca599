"""The schedule of the MIC(0) triangular solves (csrc/pressure.cu, k_tri and
k_tri_cl), restated on the CPU: which block a CTA of a cluster owns, which
thread hands which edge value to which receive slot, and how the input ring's
copy groups are waited for.  Host-side checks of the kernels' index arithmetic,
no GPU involved:

- every remote store into a receive buffer and every receive read is in
  bounds, and every read is matched by exactly one store from the block
  upstream (so no wait can be left without its value), for ragged grids, blocks
  without fluid, both sweep directions and both cluster shapes;
- a ring slot holds the step that reads it, its copy group has completed before
  the barrier that precedes the read, and it is refilled only after its last
  read;
- the receiver warp's shared ring and the gate (L2 hand-overs): no slot is
  overwritten before it is read, every read finds its own step, and no wait is
  left without its value, under random producer and load timing.

The wavefront itself follows pressuresolver.cpp:304-386 (forward / backward
solve); its numerics are checked on the GPU against the oracle.
"""
import itertools
import random

import pytest

SBJ = SBK = 16          # pencil block (csrc/pressure.cu SBJ, SBK)
SPLANE = SBJ * SBK


def cluster_schedule(nx, ny, nz, cj_n, ck_n, bwd, w, fluid_frac, seed):
    """k_tri_cl's edge hand-overs inside clusters; returns (reads, stores)."""
    rnd = random.Random(seed)
    nbj, nbk = -(-ny // SBJ), -(-nz // SBK)
    s_planes = nx + SBJ + SBK - 2
    nr = s_planes - (SBJ - 1)                         # rx_steps
    blkf = [1 if rnd.random() < fluid_frac else 0 for _ in range(nbj * nbk)]
    ncj, nck = -(-nbj // cj_n), -(-nbk // ck_n)

    def fluid(j, k):
        q = k * nbj + j
        assert 0 <= q < nbj * nbk
        return blkf[q]

    stores, reads = {}, []
    for t in range(ncj * nck):                        # one ticket per cluster
        cj, ck = t % ncj, t // ncj
        if bwd:
            cj, ck = ncj - 1 - cj, nck - 1 - ck
        j0, k0 = cj * cj_n, ck * ck_n
        for rank in range(cj_n * ck_n):
            bj, bk = j0 + rank % cj_n, k0 + rank // cj_n
            exists = bj < nbj and bk < nbk
            live = exists and fluid(bj, bk) != 0
            pbj, pbk = (bj + 1, bk + 1) if bwd else (bj - 1, bk - 1)
            cbj, cbk = (bj - 1, bk - 1) if bwd else (bj + 1, bk + 1)
            has_pj = exists and 0 <= pbj < nbj and fluid(pbj, bk)
            has_pk = exists and 0 <= pbk < nbk and fluid(bj, pbk)
            has_cj = exists and 0 <= cbj < nbj and fluid(cbj, bk)
            has_ck = exists and 0 <= cbk < nbk and fluid(bj, cbk)
            pj_cl, pk_cl = j0 <= pbj < j0 + cj_n, k0 <= pbk < k0 + ck_n
            cj_cl, ck_cl = j0 <= cbj < j0 + cj_n, k0 <= cbk < k0 + ck_n
            for tid in range(SPLANE):
                jl, kl = tid % SBJ, tid // SBJ
                valid = live and bj * SBJ + jl < ny and bk * SBK + kl < nz
                at_j = jl == SBJ - 1 if bwd else jl == 0
                at_k = kl == SBK - 1 if bwd else kl == 0
                out_j = (jl == 0 if bwd else jl == SBJ - 1) and has_cj
                out_k = (kl == 0 if bwd else kl == SBK - 1) and has_ck
                st_lo = (s_planes - nx - jl - kl if bwd else jl + kl) if valid else s_planes
                st_hi = st_lo + nx if valid else s_planes
                for st in range(st_lo, min(st_hi, s_planes)):
                    if at_j and has_pj and pj_cl:
                        idx = (st * SBK + kl) * w
                        assert 0 <= idx and idx + w <= nr * SBK * w
                        reads.append(((bj, bk), "j", idx, (pbj, bk)))
                    if at_k and has_pk and pk_cl:
                        idx = (st * SBJ + jl) * w
                        assert 0 <= idx and idx + w <= nr * SBJ * w
                        reads.append(((bj, bk), "k", idx, (bj, pbk)))
                    if out_j and cj_cl:
                        assert 0 <= rank + (cbj - bj) < cj_n * ck_n
                        idx = (kl + (st - (SBJ - 1)) * SBK) * w
                        assert 0 <= idx and idx + w <= nr * SBK * w
                        key = ((cbj, bk), "j", idx)
                        assert key not in stores
                        stores[key] = (bj, bk)
                    if out_k and ck_cl:
                        assert 0 <= rank + (cbk - bk) * cj_n < cj_n * ck_n
                        idx = (jl + (st - (SBK - 1)) * SBJ) * w
                        assert 0 <= idx and idx + w <= nr * SBJ * w
                        key = ((bj, cbk), "k", idx)
                        assert key not in stores
                        stores[key] = (bj, bk)
    return reads, stores


@pytest.mark.parametrize("dims", [(40, 37, 23), (16, 16, 16), (17, 33, 50), (30, 129, 65)])
@pytest.mark.parametrize("shape", [(4, 2), (2, 2)])
@pytest.mark.parametrize("bwd", [False, True])
def test_cluster_handovers_match(dims, shape, bwd):
    for w, frac in ((1, 1.0), (2, 0.6)):
        reads, stores = cluster_schedule(*dims, *shape, bwd, w, frac, seed=sum(dims))
        for blk, edge, idx, producer in reads:
            assert stores.get((blk, edge, idx)) == producer, (blk, edge, idx)


def ring_schedule(s_planes, p):
    """The input ring: P copy groups in flight, a slot refilled one step after
    its last read, wait_group<P-2> before each step's barrier."""
    done, slot = [], {}

    def commit(items):
        done.append(False)
        for sl, step in items:
            slot[sl] = (step, len(done) - 1)

    def wait(n):
        for g in range(len(done) - n):
            done[g] = True

    for u in range(p):
        commit([(u, u)] if u < s_planes else [])
    wait(p - 1)
    visible = {sl: v for sl, v in slot.items() if done[v[1]]}
    last_read = {}
    for st in range(-(-s_planes // p) * p):
        u = st % p
        items = []
        if st >= 1 and st - 1 + p < s_planes:
            sl = (u + p - 1) % p
            assert last_read.get(sl) == st - 1
            items.append((sl, st - 1 + p))
        commit(items)
        if st < s_planes:
            step, g = visible[u]
            assert step == st and done[g]
            last_read[u] = st
        wait(p - 2)
        visible = {sl: v for sl, v in slot.items() if done[v[1]]}


@pytest.mark.parametrize("p", [4, 8])
def test_ring_refill_order(p):
    for s_planes in itertools.chain(range(1, 40), (286, 301, 542)):
        ring_schedule(s_planes, p)


# ----------------------------------------------------------------------------
# The receiver warps and the gate (csrc/pressure.cu rx_receive, rx_gate, k_tri):
# a discrete-time restatement with random producer and load timing.  Lane l of
# receiver class r takes the steps s = r (mod RX_NR) of edge pencil l with one read
# in flight: each tick it issues the read of its next step if that step is within
# room = max(cons, lo) + RX_R - RX_CB, or, once its read has seen the word,
# publishes it into ring slot s % RX_R and moves on by RX_NR, or reissues the read.
# The compute threads run step st once the gate has seen, for every lane active at
# st, the minimum progress over the classes past st; they read ring slot st % RX_R
# and every RX_CB steps hand back the slots below st.  Checked: no slot is written
# while it holds a step not yet read, every read finds its own step's value, and the
# sweep ends within a bounded number of ticks (no circular wait), for lanes with
# different active ranges (forward and backward) and lanes without a producer.

RX_R, RX_NR, RX_CB = 32, 4, 8
DONE = 1 << 30


def rx_emulate(s_planes, lanes, seed):
    """lanes: list of (lo, hi) active step ranges, or None for a lane without a
    producer.  Returns the number of ticks the sweep took."""
    rnd = random.Random(seed)
    # the producer's word of step s (for lane l) becomes visible at tick avail[l][s]
    avail = []
    for rng in lanes:
        a = {}
        if rng is not None:
            t = rnd.randrange(0, 6)
            for s in range(rng[0], rng[1]):
                t += rnd.choice((0, 0, 1, 1, 2, 5))
                a[s] = t
        avail.append(a)
    ring = {}                   # slot -> (lane -> step it holds)
    prog = [[0] * RX_NR for _ in lanes]
    cons = 0
    cl = []                     # per lane, per class: [next step, read in flight, tick it was issued]
    for l, rng in enumerate(lanes):
        if rng is None:
            cl.append(None)
            continue
        lo, hi = rng
        row = []
        for r in range(RX_NR):
            s0 = lo + (r - lo) % RX_NR
            row.append([s0, False, 0])
            prog[l][r] = s0 if s0 < hi else DONE
        cl.append(row)
    tick, st = 0, 0
    limit = 50 * (s_planes + 100)
    while st < s_planes:
        tick += 1
        assert tick < limit, "the sweep did not finish: a wait that never ends"
        for l, rng in enumerate(lanes):
            if cl[l] is None:
                continue
            lo, hi = rng
            room = max(cons, lo) + RX_R - RX_CB
            for r in range(RX_NR):
                c = cl[l][r]
                s = c[0]
                if s >= hi:
                    continue
                if not c[1]:
                    if s < room:
                        c[1], c[2] = True, tick
                elif avail[l][s] <= c[2]:                  # the read saw the word
                    slot = s % RX_R
                    held = ring.setdefault(slot, {}).get(l)
                    assert held is None or held < cons, (l, s, held, cons)   # its step was read
                    ring[slot][l] = s
                    s += RX_NR
                    c[0], c[1] = s, False
                    prog[l][r] = s if s < hi else DONE
                    if s < hi and s < room:
                        c[1], c[2] = True, tick
                else:
                    c[2] = tick                            # reissue
        # compute: step st runs once the gate has seen every active lane's input of st
        if all(rng is None or not (rng[0] <= st < rng[1]) or min(prog[l]) > st for l, rng in enumerate(lanes)):
            for l, rng in enumerate(lanes):
                if rng is not None and rng[0] <= st < rng[1]:
                    assert ring[st % RX_R][l] == st, (l, st, ring[st % RX_R].get(l))
            if ((st + 1) % RX_CB) == 0:
                cons = st                                  # steps below st have been read
            st += 1
    return tick


@pytest.mark.parametrize("bwd", [False, True])
def test_receiver_ring_and_gate(bwd):
    for nx, seed in itertools.product((1, 5, 40, 100, 256), range(4)):
        s_planes = nx + SBJ + SBK - 2
        lanes = []
        for lane in range(32):
            e, idx = lane >> 4, lane & 15
            jl, kl = (SBJ - 1 if bwd else 0, idx) if e == 0 else (idx, SBK - 1 if bwd else 0)
            if (lane * 7 + seed) % 9 == 0:
                lanes.append(None)                         # no producer on this edge pencil
                continue
            lo = s_planes - nx - jl - kl if bwd else jl + kl
            lanes.append((lo, lo + nx))
        ticks = rx_emulate(s_planes, lanes, seed)
        assert ticks >= s_planes
