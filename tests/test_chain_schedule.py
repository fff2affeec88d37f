"""The schedule of the chained exact-order SOR (k_sor_chain), checked on the
CPU: a step-by-step model of what each row does, with the kernel's own pass
cursor, against the order that compute_flow's lexicographic sweeps impose
(core/level_solver.py:257-364).

For every level shape and pass list below it checks that
* every (pass, iteration, pixel) is updated exactly once, at step
  s = r + start_p + c + 2 gi, and a row never works on two passes at once;
* every value an update reads is the right version: the row above and the
  column to the left at this iteration one step earlier (shuffles and
  registers), the row below and the column to the right at the previous
  iteration one step earlier, the pixel itself two steps earlier; at a pass
  start, the previous pass's final value, stored strictly before the
  prefetch that loads it (a later step than the store, and for the row below
  at least one barrier later) and overwritten only after it;
* a pixel's folded coefficients stay in their ring slot from the fold to the
  last update that reads them.
The GPU tests check that the kernel gives the same bits as one launch per
pass; this model shows why it can.
"""
import pytest


def passes_model(iterations, lag, gmax):
    """(G, mode) per wavefront pass, as make_passes in frg_api.cu."""
    starts = [0] + [t for t in range(1, iterations) if (t + 1) % lag == 0]
    out = []
    for i, s in enumerate(starts):
        e = starts[i + 1] if i + 1 < len(starts) else iterations
        mode = (1 if s == 0 else 0) | (2 if (s + 1) % lag == 0 else 0)
        for q in range(s, e, gmax):
            out.append((min(gmax, e - q), mode if q == s else -1))
    return out


def span(w, g):
    return w + (2 * (g - 1) if g > 1 else 1)


def simulate(h, w, Gs):
    """Replays k_sor_chain's cursor and step loop; returns the update step of
    every (pass, gi, r, c), the prefetch step of every (pass, r, c) entering
    pixel and of every (pass, r, c) "pixel below" load, and the fold step of
    every entering pixel."""
    gmax = max(Gs)
    starts, s0 = [], 0
    for g in Gs:
        starts.append(s0)
        s0 += span(w, g)
    nsteps = s0 + h - 1
    last = len(Gs) - 1
    upd, fetch_raw, fetch_below, fold = {}, {}, {}, {}
    for r in range(h):
        cp, cstart, cend = 0, 0, span(w, Gs[0])

        def where(tau):
            # the pass the fold (tau + 1) or prefetch (tau + 2) falls in: current or next
            if cp < last and tau >= cend:
                return cp + 1, tau - cend
            return cp, tau - cstart

        # before the loop: the prefetch of local times -r and 1 - r (as if at steps -2
        # and -1) and the fold of -r (as if at step -1)
        for tau, at in ((-r, -2), (1 - r, -1)):
            p, c = where(tau)
            if 0 <= c < w:
                fetch_raw[(p, r, c)] = at
            if 1 <= c <= w and r + 1 < h:
                fetch_below[(p, r + 1, c - 1)] = at
        p, c = where(-r)
        if 0 <= c < w:
            fold[(p, r, c)] = -1
        for s in range(nsteps):
            tau = s - r
            if tau >= cend and cp < last:
                cp += 1
                cstart = cend
                cend = cstart + span(w, Gs[cp])
            active = []
            for gi in range(gmax):
                c = tau - cstart - 2 * gi
                if gi < Gs[cp] and 0 <= c < w:
                    active.append((cp, gi, c))
            assert len({a[0] for a in active}) <= 1
            p, c = where(tau + 2)
            if 0 <= c < w:
                fetch_raw[(p, r, c)] = s
            if 1 <= c <= w and r + 1 < h:
                fetch_below[(p, r + 1, c - 1)] = s
            for (p_, gi, c_) in active:
                key = (p_, gi, r, c_)
                assert key not in upd
                upd[key] = s
            p, c = where(tau + 1)
            if 0 <= c < w:
                fold[(p, r, c)] = s
    return starts, upd, fetch_raw, fetch_below, fold


SHAPES = [(1, 3), (2, 3), (5, 4), (7, 9), (33, 40), (40, 33), (64, 5)]
SCHEDULES = [(50, 5, 5), (20, 5, 3), (20, 5, 1), (12, 4, 2), (9, 3, 5), (7, 1, 5), (11, 6, 4)]


@pytest.mark.parametrize("h,w", SHAPES)
@pytest.mark.parametrize("iterations,lag,gmax", SCHEDULES)
def test_chained_schedule_keeps_lexicographic_order(h, w, iterations, lag, gmax):
    Gs = [g for g, _ in passes_model(iterations, lag, gmax)]
    starts, upd, fetch_raw, fetch_below, fold = simulate(h, w, Gs)
    S = 2 * max(Gs) - 1
    # every update once, at its formula step
    assert len(upd) == sum(Gs) * h * w
    for (p, gi, r, c), s in upd.items():
        assert s == r + starts[p] + c + 2 * gi

    def final(p, r, c):  # step that stores pass p's final value of (r, c)
        return upd[(p, Gs[p] - 1, r, c)]

    for (p, gi, r, c), s in upd.items():
        if r > 0:
            assert upd[(p, gi, r - 1, c)] == s - 1  # above, this iteration
        if c > 0:
            assert upd[(p, gi, r, c - 1)] == s - 1  # left, this iteration
        if gi > 0:
            assert upd[(p, gi - 1, r, c)] == s - 2  # itself, previous iteration
            if r + 1 < h:
                assert upd[(p, gi - 1, r + 1, c)] == s - 1  # below, previous iteration
            if c + 1 < w:
                assert upd[(p, gi - 1, r, c + 1)] == s - 1  # right, previous iteration
            continue
        # pass start: itself and its right neighbour come from this row's prefetch, the
        # row below from this row's "below" prefetch; the previous pass stored them first
        assert fetch_raw[(p, r, c)] == s - 2
        if c + 1 < w:
            assert fetch_raw[(p, r, c + 1)] == s - 1
        if r + 1 < h:
            assert fetch_below[(p, r + 1, c)] == s - 1
        if p > 0:
            assert final(p - 1, r, c) < fetch_raw[(p, r, c)]
            if c + 1 < w:
                assert final(p - 1, r, c + 1) < fetch_raw[(p, r, c + 1)]
            if r + 1 < h:
                assert final(p - 1, r + 1, c) + 1 <= fetch_below[(p, r + 1, c)]
        # nothing overwrites them before they are read
        assert fetch_raw[(p, r, c)] < final(p, r, c)
        if r + 1 < h:
            assert fetch_below[(p, r + 1, c)] < final(p, r + 1, c)
    # coefficients: folded the step before the pixel enters, into slot (entry step) mod S;
    # the next fold into that slot comes after the pixel's last read
    entries = {}
    for (p, r, c), s in fold.items():
        e = r + starts[p] + c
        assert s == e - 1
        entries.setdefault(r, []).append((e, p))
    for r, es in entries.items():
        es.sort()
        for i, (e, p) in enumerate(es):
            last_read = e + 2 * (Gs[p] - 1)
            for e2, _ in es[i + 1:]:
                if e2 % S == e % S:
                    # the overwrite happens at step e2 - 1, after that step's reads
                    assert e2 - 1 >= last_read
                    break
