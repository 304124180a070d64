"""Host model of the windowed merge carry-out (sbp_gb300/csrc/carry.cu) against the
reference's one-at-a-time queue loop (src/block_merge.cpp:54-95).

The device evaluates the W smallest live entries against one blockmodel state and replays
the pop / put-back / merge rule over those values.  This model applies the same selection,
replay and put-back buffering (shared buffer of capacity QS spilling into a sorted run)
with a stand-in for the recomputed delta that changes whenever a merge changes the state,
and must produce exactly the sequential loop's merges, in order.

Two models of the warp-level replays follow: the carry-out's put-back list in lane
registers against the single-thread insertion sort, and the MH chain window's one-ballot
stop (sbp_gb300/csrc/chain_window.cu) against the serial replay."""
import heapq
import random

import pytest


def _instance(seed, B):
    rng = random.Random(seed)
    best = [rng.randrange(B) for _ in range(B)]
    for i in range(B):
        if best[i] == i:
            best[i] = (i + 1) % B
    # integer-valued deltas make ties common
    d0 = [rng.choice([rng.uniform(-5, 5), float(rng.randrange(-3, 3))]) for _ in range(B)]
    return best, d0


def _recomputed(frm, to, version, seed):
    r = random.Random(hash((frm, to, version, seed)))
    return r.choice([r.uniform(-6, 6), float(r.randrange(-3, 4))])


def _find(parent, x):
    while parent[x] != x:
        x = parent[x]
    return x


def _sequential(best, d0, ntm, seed):
    q = [(d0[i], i) for i in range(len(best))]
    heapq.heapify(q)
    parent = list(range(len(best)))
    version, merges = 0, []
    while len(merges) < ntm and q:
        _, frm = heapq.heappop(q)
        to = _find(parent, best[frm])
        if to == frm:
            continue
        act = _recomputed(frm, to, version, seed)
        if q and act > q[0][0]:
            heapq.heappush(q, (act, frm))
            continue
        parent[frm] = to
        version += 1
        merges.append((frm, to))
    return merges


def _windowed(best, d0, ntm, seed, W, QS):
    P = sorted((d0[i], i) for i in range(len(best)))
    p, R, q, S = 0, [], 0, []
    parent = list(range(len(best)))
    version, merges = 0, []
    while len(merges) < ntm:
        heads = [P[p:p + W + 1], R[q:q + W + 1], S[:W + 1]]
        items = sorted((it, src) for src in range(3) for it in heads[src])
        ncand = min(W, len(items))
        if ncand == 0:
            break
        cands = items[:ncand]
        bound = items[W][0] if len(items) > W else None
        evals = []
        for (_, frm), _src in cands:
            to = _find(parent, best[frm])
            evals.append((to, _recomputed(frm, to, version, seed) if to != frm else None))
        i, Q, cons, mf = 0, [], [0, 0, 0], None
        while True:
            pick = None
            if i < ncand:
                pick = ("c", cands[i][0])
            if Q and (pick is None or (Q[0][0], Q[0][1]) < pick[1]):
                pick = ("q", (Q[0][0], Q[0][1]))
            if pick is None or (bound is not None and bound < pick[1]):
                break
            if pick[0] == "q":
                mf = (Q[0][1], Q[0][2])
                Q.pop(0)
                break
            (_, frm), src = cands[i]
            to, act = evals[i]
            cons[src] += 1
            i += 1
            if to == frm:
                continue
            heads_left = [x for x in (bound[0] if bound else None, cands[i][0][0] if i < ncand else None,
                                      Q[0][0] if Q else None) if x is not None]
            if heads_left and act > min(heads_left):
                Q.append((act, frm, to))
                Q.sort()
                continue
            mf = (frm, to)
            break
        p += cons[0]
        q += cons[1]
        S = sorted(S[cons[2]:] + [(a, f) for a, f, _t in Q])
        if len(S) > QS - W - 1:
            R, q, S = sorted(R[q:] + S), 0, []
        if mf:
            parent[mf[0]] = mf[1]
            version += 1
            merges.append(mf)
    return merges


@pytest.mark.parametrize("W,QS", [(1, 8), (3, 12), (16, 40), (16, 1024)])
def test_windowed_carry_out_matches_sequential_queue(W, QS):
    for seed in range(150):
        B = random.Random(seed).randrange(2, 250)
        best, d0 = _instance(seed, B)
        ntm = random.Random(seed + 1).randrange(1, B)
        assert _windowed(best, d0, ntm, seed, W, QS) == _sequential(best, d0, ntm, seed), (seed, B)


# ---- the carry-out's replay on one warp (carry.cu, step 3): the round's put-back list
# lives in lane registers, entry l in lane l.  These model the warp primitives with the
# kernel's own lane arithmetic and check them against the sorted list the single-thread
# replay kept (an insertion sort on (delta, block), pops from the front).

def _qless(a, b):
    return a[0] < b[0] or (a[0] == b[0] and a[1] < b[1])


def _shfl_down(lanes, delta):
    return [lanes[l + delta] if l + delta < 32 else lanes[l] for l in range(32)]


def _shfl_up(lanes, delta):
    return [lanes[l - delta] if l - delta >= 0 else lanes[l] for l in range(32)]


def _warp_pop(lanes):
    return _shfl_down(lanes, 1)


def _warp_insert(lanes, nq, new):
    """k = popc(ballot(lane < nq && qless(q[lane], new))); lanes above k take their lower
    neighbour's entry, lane k the new one."""
    k = sum(1 for l in range(32) if l < nq and _qless(lanes[l], new))
    up = _shfl_up(lanes, 1)
    return [up[l] if l > k else (new if l == k else lanes[l]) for l in range(32)]


def _thread_insert(q, new):
    q = list(q)
    k = len(q)
    q.append(None)
    while k > 0 and _qless(new, q[k - 1]):
        q[k] = q[k - 1]
        k -= 1
    q[k] = new
    return q


@pytest.mark.parametrize("seed", range(40))
def test_warp_put_back_list_matches_insertion_sort(seed):
    rng = random.Random(seed)
    lanes = [(0, -1)] * 32
    ref, nq = [], 0
    blocks = rng.sample(range(1000), 64)  # a block is in the list at most once
    for step in range(200):
        if nq > 0 and (nq == 16 or rng.random() < 0.45):
            assert lanes[0] == ref[0]
            lanes = _warp_pop(lanes)
            ref.pop(0)
            nq -= 1
        else:
            free = [b for b in blocks if all(b != e[1] for e in ref)]
            new = (rng.choice([rng.randrange(-3, 3), rng.uniform(-3, 3)]), rng.choice(free))
            lanes = _warp_insert(lanes, nq, new)
            ref = _thread_insert(ref, new)
            nq += 1
        assert lanes[:nq] == ref, (seed, step)


# ---- the MH chain window's replay (chain_window.cu): bit u of conf[j] is set only for an
# accepted entry u < j whose move may change entry j.  The single-thread replay walked the
# entries, keeping each while no accepted earlier entry conflicts with it; the warp replay
# stops at the first entry with any bit set (one ballot).  Both keep the same entries.

def _serial_stop(conf, accepted, wn):
    consumed, acc_mask = 0, 0
    for j in range(wn):
        if conf[j] & acc_mask:
            break
        consumed = j + 1
        if accepted[j]:
            acc_mask |= 1 << j
    return consumed, acc_mask


def _ballot_stop(conf, accepted, wn):
    stop = [j for j in range(wn) if conf[j] != 0]
    consumed = stop[0] if stop else wn
    acc_mask = sum(1 << j for j in range(consumed) if accepted[j])
    return consumed, acc_mask


@pytest.mark.parametrize("seed", range(20))
def test_chain_window_ballot_stop_matches_serial_replay(seed):
    rng = random.Random(seed)
    for _ in range(500):
        wn = rng.randrange(1, 17)
        accepted = [rng.random() < rng.choice([0.1, 0.5, 0.9]) for _ in range(wn)]
        p = rng.choice([0.05, 0.3, 0.8])
        conf = [sum(1 << u for u in range(j) if accepted[u] and rng.random() < p) for j in range(wn)]
        assert _ballot_stop(conf, accepted, wn) == _serial_stop(conf, accepted, wn)


# ---- the cluster carry-out's greedy replay (sbp_gb300/csrc/carry_cluster.cu): the
# parallel first pass plus the single-thread continuation against the single-thread replay
# alone, on random rounds with ties, put-backs that pop again, stale candidates and the
# merge limit.

def _qless(a, b):
    return a < b  # (delta, block) pairs compare lexicographically


def _replay_seq(c, st):
    """The single-thread replay from state st = (i, nm, pend ranks, stl set)."""
    n, hb, bound, need = c["n"], c["hb"], c["bound"], c["need"]
    keys, act, blk, to, inv, rank = c["keys"], c["act"], c["blk"], c["to"], c["inv"], c["rank"]
    by_rank = sorted(range(n), key=lambda j: (act[j], blk[j]))
    i, merges, pend, stl = st
    merges, pend, stl = list(merges), set(pend), set(stl)
    while len(merges) < need:
        hc, hq = i < n, bool(pend)
        if not hc and not hq:
            break
        if hq:
            r = min(pend)
            q = (act[by_rank[r]], blk[by_rank[r]])
        fromq = hq and (not hc or _qless(q, keys[i]))
        k = q if fromq else keys[i]
        if hb and _qless(bound, k):
            break
        if fromq:
            ci = by_rank[r]
            if ci in stl:
                break
            pend.discard(r)
            merges.append((blk[ci], to[ci]))
            stl |= inv[ci]
            continue
        if i in stl:
            break
        ci = i
        i += 1
        if to[ci] == blk[ci]:
            continue
        hc2, hq = i < n, bool(pend)
        if hc2 or hq or hb:
            top = bound[0] if hb else float("inf")
            if hc2:
                top = min(top, keys[i][0])
            if hq:
                top = min(top, act[by_rank[min(pend)]])
            if act[ci] > top:
                pend.add(rank[ci])
                continue
        merges.append((blk[ci], to[ci]))
        stl |= inv[ci]
    return i, merges, pend, stl


def _replay_parallel(c):
    """The device's parallel first pass, then the single-thread loop from where it stopped."""
    n, hb, bound, need = c["n"], c["hb"], c["bound"], c["need"]
    keys, act, blk, to, inv, rank = c["keys"], c["act"], c["blk"], c["to"], c["inv"], c["rank"]
    same = [to[i] == blk[i] for i in range(n)]
    T0 = []
    for i in range(n):
        t = bound[0] if hb else float("inf")
        if i + 1 < n:
            t = min(t, keys[i + 1][0])
        T0.append(t)
    pb = [not same[i] and (i + 1 < n or hb) and act[i] > T0[i] for i in range(n)]
    mg = [not same[i] and not pb[i] for i in range(n)]
    P, S, L = n, n, (1 << 30) if need > 0 else 0
    qmin, before, ex = None, 0, set()
    for i in range(n):
        if qmin is not None and not (qmin[0] >= T0[i] and not _qless(qmin, keys[i])):
            P = min(P, i)
        if i in ex:
            S = min(S, i)
        if mg[i] and before == need - 1:
            L = min(L, i + 1)
        if pb[i] and (qmin is None or _qless((act[i], blk[i]), qmin)):
            qmin = (act[i], blk[i])
        if mg[i]:
            before += 1
            ex |= inv[i]
    end = min(P, S, L)
    merges, pend, stl = [], set(), set()
    for i in range(end):
        if mg[i]:
            merges.append((blk[i], to[i]))
            stl |= inv[i]
        if pb[i]:
            pend.add(rank[i])
    if end == P and end < L:
        return _replay_seq(c, (end, merges, pend, stl))
    return end, merges, pend, stl


def _round(seed):
    rng = random.Random(seed)
    n = rng.randint(1, 40)
    hb = rng.random() < 0.7
    vals = sorted((rng.randrange(-6, 6), b) for b in rng.sample(range(1000), n + 1))
    keys, bound = vals[:n], vals[n]
    blk = [k[1] for k in keys]
    act = [k[0] + rng.choice([0, 0, 1, 2, -1, rng.randrange(-3, 8)]) for k in keys]
    to = [b if rng.random() < 0.1 else rng.randrange(1000, 2000) for b in blk]
    inv = [set(j for j in range(n) if j != i and rng.random() < rng.choice([0.0, 0.02, 0.1])) for i in range(n)]
    order = sorted(range(n), key=lambda j: (act[j], blk[j]))
    rank = [0] * n
    for r, j in enumerate(order):
        rank[j] = r
    need = rng.choice([n + 5, rng.randint(0, n)])
    return dict(n=n, hb=hb, bound=bound, need=need, keys=keys, act=act, blk=blk, to=to, inv=inv, rank=rank)


def test_parallel_replay_equals_single_thread():
    for seed in range(6000):
        c = _round(seed)
        want = _replay_seq(c, (0, [], set(), set()))
        got = _replay_parallel(c)
        assert got[0] == want[0] and got[1] == want[1] and got[2] == want[2], seed
