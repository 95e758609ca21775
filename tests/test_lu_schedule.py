"""Host-only check of the blocked LU's launch schedule (mpdok_lu_schedule).

The factorization issues its kernels on four streams (the caller's, a chain
stream for the work inside the current super-panel, and two streams for the
rows and columns past it) that only events order.  This test rebuilds the
happens-before relation of the exported schedule with vector clocks and checks:

* every pair of launches that touch the same data with at least one write is
  ordered.  The data are the working matrix W, the factor, the diagonal-block
  inverses, and the double-buffered L21 / U12 operands;
* every 128 x 128 block of W receives each earlier panel's update exactly once,
  and all of them before the launch that factors the block or solves with it;
* every operand an update reads was written, before it, by the panel solve of
  the same super-panel.  An earlier super-panel's write to the same buffer
  comes before it, and a later one (two super-panels on) after it.

A schedule with one of its event waits taken out must fail the check.  Nothing
here touches a GPU: the schedule is host data.
"""
import numpy as np
import pytest

from mpdok_gb300 import _native as N

LNB = 128
DIAG, SOLVE, UPDATE, RECORD, WAIT = 0, 1, 2, 3, 4
SETUP = -1


def _spw(fdtype):
    """The library's super-panel width: the start of the second super-panel
    of a schedule larger than any width."""
    s = N.lu_schedule(16384, fdtype)
    js = sorted({int(j) for j in s[s[:, 0] == DIAG][:, 2]})
    return js[1]


def _happens_before(steps):
    """Kernel ops (with a setup op first: the scaling and the working copy on
    the caller's stream) and a predicate hb(i, j): op i completes before op j
    starts on the GPU."""
    ns = max(3, int(steps[:, 1].max()) + 1) if len(steps) else 3
    cur = np.zeros((ns, ns), dtype=np.int64)  # vector clock of each stream
    count = [1] + [0] * (ns - 1)              # the setup op is position 1 of stream 0
    cur[0, 0] = 1
    recorded = {}
    ops = [dict(kind=SETUP, stream=0, pos=1, clock=cur[0].copy())]
    for row in steps:
        kind, st = int(row[0]), int(row[1])
        if kind == RECORD:
            recorded[int(row[11])] = cur[st].copy()
        elif kind == WAIT:
            ev = int(row[11])
            if ev in recorded:  # a wait on an event never recorded is a no-op
                cur[st] = np.maximum(cur[st], recorded[ev])
        elif kind in (DIAG, SOLVE, UPDATE):
            count[st] += 1
            cur[st, st] = count[st]
            ops.append(dict(kind=kind, stream=st, pos=count[st], clock=cur[st].copy(), row=row))

    def hb(i, j):
        return i != j and ops[j]["clock"][ops[i]["stream"]] >= ops[i]["pos"]

    return ops, hb


def _accesses(op, n, spw):
    """(resource, (r0, r1, c0, c1), writes) of one op."""
    if op["kind"] == SETUP:
        return [("W", (0, n, 0, n), True)]
    _, _, J, jp, a, b, m, nn, K, koff, rb, _ = (int(x) for x in op["row"])
    buf = (J // spw) & 1
    nbk = min(LNB, n - jp)
    blk = (jp, jp + nbk, jp, jp + nbk)
    if op["kind"] == DIAG:
        # factors the block in place (W keeps L\\U in FP32 for the panel solves)
        return [("W", blk, True), ("LU", blk, True), (("inv", jp // LNB), (0, 1, 0, 1), True)]
    if op["kind"] == SOLVE:
        slot = jp - J
        return [("W", blk, False), ("W", (a, b, jp, jp + LNB), False), ("W", (jp, jp + LNB, a, b), False),
                (("inv", jp // LNB), (0, 1, 0, 1), False),
                (("Lp", buf), (a - J, b - J, slot, slot + LNB), True),
                (("Up", buf), (a - J, b - J, slot, slot + LNB), True),
                ("LU", (a, b, jp, jp + LNB), True), ("LU", (jp, jp + LNB, a, b), True)]
    return [(("Lp", buf), (a - J, a - J + m, koff, koff + K), False),
            (("Up", buf), (b - J, b - J + nn, koff, koff + K), False),
            ("W", (a, a + m, b, b + nn), True)]


def _overlap(p, q):
    return p[0] < q[1] and q[0] < p[1] and p[2] < q[3] and q[2] < p[3]


def check_schedule(steps, n, fdtype):
    """Raise AssertionError on the first unordered conflict or misplaced update."""
    spw = _spw(fdtype)
    ops, hb = _happens_before(steps)
    acc = {}
    for i, op in enumerate(ops):
        for res, rect, wr in _accesses(op, n, spw):
            acc.setdefault(res, []).append((i, rect, wr))
    # 1. conflicting accesses are ordered
    for res, lst in acc.items():
        for x in range(len(lst)):
            i, ri, wi = lst[x]
            for y in range(x + 1, len(lst)):
                j, rj, wj = lst[y]
                if i != j and (wi or wj) and _overlap(ri, rj):
                    assert hb(i, j) or hb(j, i), f"unordered {res} access: ops {i} and {j}"
    # 2. every block gets each earlier panel once, before its consumer
    nb = (n + LNB - 1) // LNB
    applied = {}
    for i, op in enumerate(ops):
        if op["kind"] != UPDATE:
            continue
        _, _, J, _, a, b, m, nn, K, koff, _, _ = (int(x) for x in op["row"])
        assert a % LNB == 0 and b % LNB == 0 and K % LNB == 0 and koff % LNB == 0
        panels = range((J + koff) // LNB, (J + koff + K) // LNB)
        for bi in range(a // LNB, (a + m + LNB - 1) // LNB):
            for bj in range(b // LNB, (b + nn + LNB - 1) // LNB):
                applied.setdefault((bi, bj), []).extend((q, i) for q in panels)
    consumers = {}
    for i, op in enumerate(ops):
        if op["kind"] == DIAG:
            q = int(op["row"][3]) // LNB
            consumers.setdefault((q, q), []).append(i)
        elif op["kind"] == SOLVE:
            jp, a, b = (int(op["row"][k]) for k in (3, 4, 5))
            q = jp // LNB
            for blk in range(a // LNB, (b + LNB - 1) // LNB):
                consumers.setdefault((blk, q), []).append(i)
                consumers.setdefault((q, blk), []).append(i)
    for bi in range(nb):
        for bj in range(nb):
            got = sorted(q for q, _ in applied.get((bi, bj), []))
            assert got == list(range(min(bi, bj))), f"block ({bi},{bj}) got panels {got}"
            cons = consumers.get((bi, bj), [])
            assert len(cons) == 1, f"block ({bi},{bj}) has consumers {cons}"
            for _, u in applied.get((bi, bj), []):
                assert hb(u, cons[0]), f"update {u} of block ({bi},{bj}) not before its consumer {cons[0]}"
    # 3. operands: written by the same super-panel's solve before the read; an
    #    earlier super-panel's write to the buffer before it, a later one after
    for res in [r for r in acc if isinstance(r, tuple) and r[0] in ("Lp", "Up")]:
        writes = [(i, rect) for i, rect, wr in acc[res] if wr]
        for i, rect, wr in acc[res]:
            if wr:
                continue
            J = int(ops[i]["row"][2])
            covered = np.zeros((rect[1] - rect[0], rect[3] - rect[2]), dtype=bool)
            for w, wrect in writes:
                if not _overlap(rect, wrect):
                    continue
                if int(ops[w]["row"][2]) == J:
                    assert hb(w, i), f"operand read {i} before its write {w}"
                    covered[max(wrect[0], rect[0]) - rect[0]:min(wrect[1], rect[1]) - rect[0],
                            max(wrect[2], rect[2]) - rect[2]:min(wrect[3], rect[3]) - rect[2]] = True
                elif int(ops[w]["row"][2]) < J:
                    assert hb(w, i), f"operand {res}: stale write {w} after read {i}"
                else:
                    assert hb(i, w), f"operand {res} overwritten by op {w} before read {i}"
            assert covered.all(), f"operand read {i} not fully written"
        for x in range(len(writes)):
            for y in range(len(writes)):
                w1, r1 = writes[x]
                w2, r2 = writes[y]
                if int(ops[w1]["row"][2]) < int(ops[w2]["row"][2]) and _overlap(r1, r2):
                    assert hb(w1, w2), f"operand {res}: write {w2} not after the earlier super-panel's {w1}"


CASES = [(7000, N.F16), (9000, N.BF16), (4096, N.F16), (3000, N.F16), (1000, N.BF16), (1100, N.F16), (2500, N.F32),
         (300, N.F16), (129, N.F32), (128, N.F16), (1, N.F16)]


@pytest.mark.parametrize("n,fdtype", CASES)
def test_schedule_orders_every_conflict(n, fdtype):
    check_schedule(N.lu_schedule(n, fdtype), n, fdtype)


def test_schedule_has_four_streams_at_look_ahead_sizes():
    s = N.lu_schedule(7000, N.F16)
    kernels = s[np.isin(s[:, 0], [DIAG, SOLVE, UPDATE])]
    assert set(np.unique(kernels[:, 1])) == {0, 1, 2, 3}
    # the chain stream touches only rows and columns of its own super-panel,
    # except for part (a) of its far update: the next super-panel's rows and
    # columns, with K = the super-panel's width
    spw = _spw(N.F16)
    for row in kernels[kernels[:, 1] == 1]:
        J, a, b, m, nn, K = (int(row[k]) for k in (2, 4, 5, 6, 7, 8))
        Jend = min(7000, J + spw)
        if int(row[0]) == SOLVE:
            assert b <= Jend
        elif int(row[0]) == UPDATE:
            inside = a + m <= Jend and b + nn <= Jend
            cross = K == Jend - J and a >= Jend and b >= Jend and (a + m <= Jend + spw or b + nn <= Jend + spw)
            assert inside or cross
    s = N.lu_schedule(1000, N.F16)  # one super-panel: the caller's stream alone
    assert set(np.unique(s[np.isin(s[:, 0], [DIAG, SOLVE, UPDATE]), 1])) == {0}


@pytest.mark.parametrize("which", ["previous_far_update_before_cross_update", "chain_before_below_solve",
                                   "below_before_far_update", "below_solve_before_row_update"])
def test_checker_catches_a_missing_wait(which):
    """A planted mistake: drop one event wait from the exported schedule."""
    n, fd = 7000, N.F16
    s = N.lu_schedule(n, fd)
    waits = np.nonzero(s[:, 0] == WAIT)[0]
    pick = {
        # the chain stream's wait for part (b) of the previous far update
        # before it updates the next super-panel's rows and columns
        "previous_far_update_before_cross_update": [w for w in waits if s[w, 1] == 1 and s[w, 11] == 4],
        # the below stream's wait for the panel's diagonal LU and solve
        "chain_before_below_solve": [w for w in waits if s[w, 1] == 2 and s[w, 11] == 2],
        # the chain stream's join of the below stream before the far update
        "below_before_far_update": [w for w in waits if s[w, 1] == 1 and s[w, 11] == 3],
        # the second below stream's wait for the previous panel solve below
        # (whose U12 columns its row-block update reads)
        "below_solve_before_row_update": [w for w in waits if s[w, 1] == 3 and s[w, 11] == 6],
    }[which]
    assert pick
    broken = np.delete(s, pick[len(pick) // 2], axis=0)
    with pytest.raises(AssertionError):
        check_schedule(broken, n, fd)


def test_schedule_rejects_bad_arguments():
    with pytest.raises(N.MPDOKError):
        N.lu_schedule(-1, N.F16)
    with pytest.raises(N.MPDOKError):
        N.lu_schedule(100, N.F64)
