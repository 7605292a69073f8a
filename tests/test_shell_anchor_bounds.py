"""Index arithmetic of the brick bounds' shell anchors (iso.cu shell_terms), restated on the CPU
over every window the bounds form at maxDepth 8, 10 and 12: each anchor that is looked up lies in
one of the leaf's 27 neighbourhood cells (its depth-r ancestor is within one leaf of the leaf), and
every anchor-table index is in range.  (An earlier version looked up depth d-2 anchors beyond the
window; their ancestors could be two leaves away, outside the neighbour table.)"""


def _window_axis(g0, B, Lc, r, d, D):
    sh, span = D - d, 1 << (d - r)
    llo = Lc * span
    vlo = (g0 >> sh) if g0 == (llo << sh) else ((g0 - 1) >> sh)
    vhi = (g0 + B - 1) >> sh
    cross = (vlo - 1 < llo) or (vhi + 1 >= llo + span)
    return vlo - 1, vhi - vlo + 3, cross


def test_anchor_indices_stay_in_the_neighbourhood():
    checked = 0
    for D in (8, 10, 12):
        for r in range(2, D):
            S = 1 << (D - r)
            for kind in ("brick", "super"):
                E = min(S, 8) if kind == "brick" else 32
                if kind == "super" and D - r < 6:
                    continue
                nb = S // E
                for Lc in (0, 1, (1 << r) - 1):
                    for b in sorted({0, 1, nb // 2, nb - 2, nb - 1}):
                        if not 0 <= b < nb:
                            continue
                        g0 = Lc * S + b * E
                        for d in range(r + 3, D + 1):
                            wlo, ext, cross = _window_axis(g0, E, Lc, r, d, D)
                            if not cross or ext > 12:   # no shell terms, or the super-brick is undecided
                                continue
                            checked += 1
                            alo, blo = wlo >> 4, wlo >> 2
                            ahi, bhi = (wlo + ext - 1) >> 4, (wlo + ext - 1) >> 2
                            if d - r > 4:
                                for A in range(alo, min(alo + 2, ahi + 1)):
                                    assert abs((A >> (d - 4 - r)) - Lc) <= 1
                            for Bc in range(blo, min(blo + 4, bhi + 1)):
                                assert abs((Bc >> (d - 2 - r)) - Lc) <= 1
                                if d - r > 4:
                                    assert 0 <= (Bc >> 2) - alo <= 1
                            for N in range(wlo, wlo + ext):
                                assert 0 <= (N >> 2) - blo <= 3
    assert checked > 500


def test_windows_leave_the_leaf_only_at_coarse_depths():
    """The bounds stop at the first depth whose window lies inside the leaf: the windows of
    successive depths are nested, so crossing the leaf's boundary is monotone in depth."""
    n = 0
    for D in range(4, 13):
        for r in range(1, D):
            S = 1 << (D - r)
            for E in sorted({min(S, 8), 32 if S >= 64 else min(S, 8)}):
                nb = S // E
                for Lc in range(min(1 << r, 4)):
                    for b in range(nb):
                        crosses = [_window_axis(Lc * S + b * E, E, Lc, r, d, D)[2] for d in range(r + 1, D + 1)]
                        first_inside = crosses.index(False) if False in crosses else len(crosses)
                        assert not any(crosses[first_inside:])
                        n += 1
    assert n > 1000
