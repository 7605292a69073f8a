"""The oracle's cascadic solve (coarse to fine, each depth's right-hand side less the coarser
depths' solution; not the reference's independent depths), on the CPU:

  * after the solve every depth's rows of the coupled system hold,
      L_d x_d + sum_{e<d} L_{d,e} x_e = b_d,
    with the cross-depth products restated here in numpy from the full inner-product tables
    (the 27 neighbours of each ancestor), to the CG tolerance; the reference's independent
    solution does not satisfy them;
  * on a sphere the cascadic mesh lies closer to the true surface than the independent one.
"""
import numpy as np

from conftest import sphere


def _coords(key, d, D):
    key = key.astype(np.int64) >> (3 * (D - d))
    p = np.zeros((len(key), 3), np.int64)
    for l in range(d - 1, -1, -1):
        for a, sh in enumerate((2, 1, 0)):
            p[:, a] = (p[:, a] << 1) | ((key >> (3 * l + sh)) & 1)
    return p


def _coupled_residual(o, D):
    key, parent = o.get("key"), o.get("parent").astype(np.int64)
    neighs = o.get("neighs").reshape(-1, 27).astype(np.int64)
    base, x, b = o.get("base"), o.get("x").astype(np.float64), o.get("divergence").astype(np.float64)
    st = o.get("stencil").reshape(-1, 27).astype(np.float64)
    res = (1 << (D + 1)) - 1
    dot = o.get("dot").reshape(res, res)
    d2 = o.get("d2dot").reshape(res, res)
    out = []
    for d in range(D + 1):
        nodes = np.arange(base[d], base[d + 1])
        fi = (1 << d) - 1 + _coords(key[nodes], d, D)
        lhs = np.zeros(len(nodes))
        for j in range(27):
            nb = neighs[nodes, j]
            ok = nb >= 0
            lhs[ok] += st[d, j] * x[nb[ok]]
        anc = nodes
        for e in range(d - 1, -1, -1):
            anc = parent[anc]
            for j in range(27):
                q = neighs[anc, j]
                ok = q >= 0
                fq = (1 << e) - 1 + _coords(key[q[ok]], e, D)
                t = [dot[fq[:, a], fi[ok, a]] for a in range(3)]
                dd = [d2[fq[:, a], fi[ok, a]] for a in range(3)]
                l = dd[0] * t[1] * t[2] + t[0] * dd[1] * t[2] + t[0] * t[1] * dd[2]
                lhs[ok] += l * x[q[ok]]
        out.append(np.linalg.norm(b[nodes] - lhs) / max(np.linalg.norm(b[nodes]), 1e-30))
    return np.array(out)


def test_cascadic_solution_holds_the_coupled_rows(oracle_mod):
    xyz, nrm = sphere(3000, seed=3)
    D = 5
    rel = {}
    for casc in (False, True):
        o = oracle_mod.Oracle(D, threads=4)
        o.set_points(xyz, nrm)
        o.set_cascadic(casc)
        o.reconstruct(1, 1e-7, 10000)
        rel[casc] = _coupled_residual(o, D)
    assert np.all(rel[True] < 1e-4), rel[True]
    # the independent depths ignore the coupling: their rows miss by far more
    assert np.all(rel[False][1:] > 1e-2), rel[False]


def test_cascadic_sphere_mesh_closer(oracle_mod):
    xyz, nrm = sphere(20000, seed=0)
    D = 7
    dist = {}
    for casc in (False, True):
        o = oracle_mod.Oracle(D)
        o.set_points(xyz, nrm)
        o.set_cascadic(casc)
        o.reconstruct(1, 1e-6, 10000)
        v = o.get("mesh_v").reshape(-1, 3) * o.get("scale")[0] + o.get("center")
        used = np.unique(o.get("mesh_f"))
        dist[casc] = np.abs(np.linalg.norm(v[used] - 0.5, axis=1) - 0.35)
    assert dist[True].max() < 0.02
    assert dist[True].mean() < 0.75 * dist[False].mean()
    assert np.quantile(dist[True], 0.99) < 0.75 * np.quantile(dist[False], 0.99)


def test_cascadic_needs_the_full_tables(oracle_mod):
    xyz, nrm = sphere(500, seed=1)
    o = oracle_mod.Oracle(4, threads=2)
    o.set_points(xyz, nrm)
    o.set_cascadic(True)
    o.build_octree()
    o.build_basis(False)
    o.vector_field()
    assert oracle_mod.lib().orc_solve(o._h, 1, 1e-6, 100) == -1
