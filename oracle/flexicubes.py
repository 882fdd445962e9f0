"""FlexiCubes surface extraction — CPU oracle, TEST INFRASTRUCTURE ONLY.

Restates the reference's FlexiCubes (``geo/flexicubes.py``; Shen et al.,
"Flexible Isosurface Extraction for Gradient-Based Mesh Optimization",
SIGGRAPH 2023) as vectorised torch on the CPU, in float64 by default, with
gradients by autograd.  Covered: the triangle-mesh path without ``grad_func``
(``__call__`` at ``geo/flexicubes.py:180-260``) in both quad-splitting modes,
which is what stage 2 calls every step (``training=True``,
``scene/gaussian_geo_model_mlp_flex.py:250-251``).  The tetrahedral output
and the QEF path (``grad_func``) are not restated.

Parity: PINNED.  ``tests/golden/make_flexicubes_golden.py`` runs the
reference's own class on the CPU and stores its outputs and autograd
gradients; ``tests/test_oracle_flexicubes.py`` checks this module against
them and checks the derived tables against ``geo/tables.py`` where the
reference tree is present.

The Dual Marching Cubes tables are derived here from their rule instead of
being transcribed (``derive_tables``):
* crossing edges of a case are the cube edges whose end corners differ in
  occupancy (s < 0); on a cube face with two crossing edges they join; on an
  ambiguous face (four crossing edges) the two edges around each occupied
  corner join; each connected set is one dual vertex, its edges ascending;
* dual vertices are ordered by the lowest corner of their set on the
  minority side (occupied corners when at most four are occupied, else the
  free ones), ties by the lowest corner on the other side;
* a case is re-checked (C16/C19 ambiguity) when it has exactly one
  ambiguous face and at least five occupied corners: the neighbour across
  that face is looked up and, when it is also such a case, the case is
  replaced by its complement 255 - case.
"""
from __future__ import annotations

import torch

# corner n of a cube sits at offset (n & 1, n >> 1 & 1, n >> 2 & 1)
# (geo/flexicubes.py:83-84); cube edges as corner pairs in the reference's
# numbering and orientation (geo/flexicubes.py:86-87)
CORNERS = [(n & 1, (n >> 1) & 1, (n >> 2) & 1) for n in range(8)]
CUBE_EDGES = [(0, 1), (1, 5), (4, 5), (0, 4), (2, 3), (3, 7), (6, 7), (2, 6),
              (2, 0), (3, 1), (7, 5), (6, 4)]
WEIGHT_SCALE = 0.99  # geo/flexicubes.py:75


def _faces():
    return [[n for n in range(8) if CORNERS[n][ax] == side] for ax in range(3) for side in (0, 1)]


def derive_tables():
    """(dmc [256][4][7], num_vd [256], check [256][5]) from the DMC rule.

    Same meaning as ``dmc_table``, ``num_vd_table`` and ``check_table`` used
    at ``geo/flexicubes.py:69-73``."""
    faces = _faces()
    dmc, num_vd, check = [], [], []
    for case in range(256):
        occ = [(case >> n) & 1 for n in range(8)]
        cross = [e for e, (a, b) in enumerate(CUBE_EDGES) if occ[a] != occ[b]]
        parent = {e: e for e in cross}

        def root(e):
            while parent[e] != e:
                e = parent[e]
            return e

        ambiguous = []
        for fi, f in enumerate(faces):
            fe = [e for e in cross if CUBE_EDGES[e][0] in f and CUBE_EDGES[e][1] in f]
            if len(fe) == 2:
                parent[root(fe[0])] = root(fe[1])
            elif len(fe) == 4:
                ambiguous.append(fi)
                for n in f:
                    if occ[n]:
                        a, b = [e for e in fe if n in CUBE_EDGES[e]]
                        parent[root(a)] = root(b)
        sets = {}
        for e in cross:
            sets.setdefault(root(e), []).append(e)
        minority = 1 if sum(occ) <= 4 else 0

        def key(edges):
            ends = {n for e in edges for n in CUBE_EDGES[e]}
            return (min(n for n in ends if occ[n] == minority),
                    min(n for n in ends if occ[n] != minority))

        groups = sorted((sorted(g) for g in sets.values()), key=key)
        dmc.append([g + [-1] * (7 - len(g)) for g in groups] + [[-1] * 7] * (4 - len(groups)))
        num_vd.append(len(groups))
        if len(ambiguous) == 1 and sum(occ) >= 5:
            ax, side = divmod(ambiguous[0], 2)
            off = [0, 0, 0]
            off[ax] = 1 if side else -1
            check.append([1] + off + [255 - case])
        else:
            check.append([0, 0, 0, 0, 0])
    return dmc, num_vd, check


def voxel_grid(res, lo=(-0.5, -0.5, -0.5), hi=(0.5, 0.5, 0.5), dtype=torch.float32):
    """Regular grid of ``construct_voxel_grid_v2`` (geo/flexicubes.py:133-157):
    vertices in (i, j, k) lexicographic order, cubes likewise, each as the
    indices of its eight corners."""
    if isinstance(res, int):
        res = (res, res, res)
    rx, ry, rz = res
    axes = [torch.linspace(float(lo[d]), float(hi[d]), res[d] + 1, dtype=dtype) for d in range(3)]
    gi, gj, gk = torch.meshgrid(*axes, indexing="ij")
    verts = torch.stack([gi, gj, gk], -1).reshape(-1, 3)
    i, j, k = torch.meshgrid(torch.arange(rx), torch.arange(ry), torch.arange(rz), indexing="ij")
    base = torch.stack([i, j, k], -1).reshape(-1, 1, 3)
    off = torch.tensor(CORNERS).reshape(1, 8, 3)
    ijk = base + off
    cubes = (ijk[..., 0] * (ry + 1) + ijk[..., 1]) * (rz + 1) + ijk[..., 2]
    return verts, cubes


def _interp(w0, w1, x0, x1):
    """Zero crossing of the line through (x0, w0), (x1, w1)
    (``_linear_interp``, geo/flexicubes.py:324-334)."""
    return (x0 * w1 - x1 * w0) / (w1 - w0)


def construct_cubes(vert_mask, res):
    """Cubes [n,8] whose corner-0 vertex is marked and inside the grid, in
    grid order (``construct_cubes`` of geo/flexicubes_no_adjacent.py:129-145)."""
    if isinstance(res, int):
        res = (res, res, res)
    rx, ry, rz = res
    m = torch.as_tensor(vert_mask).reshape(rx + 1, ry + 1, rz + 1).bool()[:rx, :ry, :rz]
    _, cubes = voxel_grid(res)
    return cubes[m.reshape(-1)]


def extract(x, s, cubes, res, beta=None, alpha=None, gamma=None, training=False, tables=None,
            de_ambiguity=True):
    """FlexiCubes triangle extraction (geo/flexicubes.py:180-260).

    x [N,3], s [N], cubes [C,8] (regular-grid order, or a subset of the grid's
    cubes in grid order), raw weights beta [C,12], alpha [C,8], gamma [C] or
    None.  de_ambiguity: the C16/C19 re-check (whole grid only); False is the
    no-adjacency variant's default (geo/flexicubes_no_adjacent.py:300-340).
    Returns (vertices, faces [F,3] int64, L_dev [E], surf_edges [Ne,2] int64)."""
    dmc, num_vd_t, check_t = tables or derive_tables()
    dmc = torch.tensor(dmc)
    num_vd_t = torch.tensor(num_vd_t)
    check_t = torch.tensor(check_t)
    dt = x.dtype
    res = (res, res, res) if isinstance(res, int) else tuple(res)

    # surface cubes (geo/flexicubes.py:306-315)
    occ = s < 0
    occ8 = occ[cubes]
    n_in = occ8.sum(1)
    surf = (n_in > 0) & (n_in < 8)
    if not bool(surf.any()):
        return (x.new_zeros((0, 3)), torch.zeros((0, 3), dtype=torch.long),
                x.new_zeros((0,)), torch.zeros((0, 2), dtype=torch.long))

    # weights (geo/flexicubes.py:262-280)
    C = cubes.shape[0]
    b = torch.tanh(beta) * WEIGHT_SCALE + 1 if beta is not None else torch.ones((C, 12), dtype=dt)
    a = torch.tanh(alpha) * WEIGHT_SCALE + 1 if alpha is not None else torch.ones((C, 8), dtype=dt)
    g = (torch.sigmoid(gamma) * WEIGHT_SCALE + (1 - WEIGHT_SCALE) / 2
         if gamma is not None else torch.ones((C,), dtype=dt))
    b, a, g = b[surf], a[surf], g[surf]

    # case ids with the C16/C19 fix (geo/flexicubes.py:282-322)
    sc = torch.nonzero(surf).squeeze(1)
    case = (occ8[surf].long() << torch.arange(8)).sum(1)
    if not de_ambiguity:
        return _extract_rest(x, s, cubes, occ, surf, sc, case, b, a, g, dmc, num_vd_t, training, dt)
    ijk = torch.stack([sc // (res[1] * res[2]), (sc // res[2]) % res[1], sc % res[2]], 1)
    flagged = torch.zeros(res, dtype=torch.bool)
    chk = check_t[case]
    to_check = chk[:, 0] == 1
    flagged[tuple(ijk[to_check].T)] = True
    nb = ijk + chk[:, 1:4]
    inside = ((nb >= 0) & (nb < torch.tensor(res))).all(1) & to_check
    invert = torch.zeros_like(inside)
    invert[inside] = flagged[tuple(nb[inside].T)]
    case = torch.where(invert, chk[:, 4], case)
    return _extract_rest(x, s, cubes, occ, surf, sc, case, b, a, g, dmc, num_vd_t, training, dt)


def _extract_rest(x, s, cubes, occ, surf, sc, case, b, a, g, dmc, num_vd_t, training, dt):
    """Surface edges, dual vertices, L_dev and triangles from the surface
    cubes and their cases."""
    # surface edges: unique grid edges of the surface cubes with a sign
    # change, lexicographic in (first vertex, second vertex)
    # (geo/flexicubes.py:286-304)
    e_all = cubes[surf][:, torch.tensor(CUBE_EDGES)].reshape(-1, 2)
    uniq, inv, cnt = torch.unique(e_all, dim=0, return_inverse=True, return_counts=True)
    crossing = occ[uniq].sum(1) == 1
    ranks = torch.full((uniq.shape[0],), -1, dtype=torch.long)
    ranks[crossing] = torch.arange(int(crossing.sum()))
    idx_map = ranks[inv].reshape(-1, 12)        # (surface cube, cube edge) -> surface edge or -1
    counts = cnt[inv].reshape(-1, 12)
    surf_edges = uniq[crossing]

    # dual vertices (geo/flexicubes.py:386-478, the branch without grad_func)
    ex = x[surf_edges]                           # [Ne,2,3]
    es = s[surf_edges]                           # [Ne,2]
    zc = _interp(es[:, 0:1], es[:, 1:2], ex[:, 0], ex[:, 1])
    nvd = num_vd_t[case]
    ent_vd, ent_cube, ent_edge = [], [], []
    vd_gamma = []
    vd_of = torch.full((sc.shape[0], 12), -1, dtype=torch.long)
    total = 0
    for num in torch.unique(nvd).tolist():
        cubes_n = torch.nonzero(nvd == num).squeeze(1)
        groups = dmc[case[cubes_n], :num]        # [n, num, 7]
        vd_ids = total + torch.arange(cubes_n.shape[0] * num).reshape(-1, num, 1).expand(-1, -1, 7)
        owner = cubes_n.reshape(-1, 1, 1).expand(-1, num, 7)
        m = groups != -1
        ent_vd.append(vd_ids[m])
        ent_cube.append(owner[m])
        ent_edge.append(groups[m])
        vd_gamma.append(g[cubes_n].repeat_interleave(num))
        total += cubes_n.shape[0] * num
    ent_vd, ent_cube, ent_edge = torch.cat(ent_vd), torch.cat(ent_cube), torch.cat(ent_edge)
    vd_gamma = torch.cat(vd_gamma)
    vd_of[ent_cube, ent_edge] = ent_vd

    se = idx_map[ent_cube, ent_edge]             # surface edge of each entry
    ce = torch.tensor(CUBE_EDGES)[ent_edge]      # its corners in the cube
    w0 = es[se, 0] * a[ent_cube, ce[:, 0]]
    w1 = es[se, 1] * a[ent_cube, ce[:, 1]]
    ue = _interp(w0.unsqueeze(1), w1.unsqueeze(1), ex[se, 0], ex[se, 1])
    bw = b[ent_cube, ent_edge].unsqueeze(1)
    bsum = torch.zeros((total, 1), dtype=dt).index_add(0, ent_vd, bw)
    vd = torch.zeros((total, 3), dtype=dt).index_add(0, ent_vd, ue * bw) / bsum
    # L_dev: mean absolute deviation of the distances from the dual vertex
    # to its unweighted zero crossings (geo/flexicubes.py:253-260)
    dist = torch.linalg.vector_norm(zc[se] - vd[ent_vd], dim=-1)
    nent = torch.zeros((total,), dtype=dt).index_add(0, ent_vd, torch.ones_like(dist))
    mean = torch.zeros((total,), dtype=dt).index_add(0, ent_vd, dist) / nent
    L_dev = (dist - mean[ent_vd]).abs()

    # quads around surface edges shared by four cubes, ordered by surface
    # edge and, within one, by cube; winding towards positive s
    # (geo/flexicubes.py:480-525)
    sel = (counts == 4) & (idx_map >= 0)
    q_edge = idx_map[sel]
    q_vd = vd_of[sel]
    order = torch.sort(q_edge, stable=True).indices
    q_edge = q_edge[order].reshape(-1, 4)[:, 0]
    quads = q_vd[order].reshape(-1, 4)
    flip = s[surf_edges[q_edge, 0]] > 0
    quads = torch.cat([quads[flip][:, [0, 1, 3, 2]], quads[~flip][:, [2, 3, 1, 0]]])
    qg = vd_gamma[quads]
    g02 = qg[:, 0] * qg[:, 2]
    g13 = qg[:, 1] * qg[:, 3]
    if not training:
        split1 = torch.tensor([0, 1, 2, 0, 2, 3])
        split2 = torch.tensor([0, 1, 3, 3, 1, 2])
        faces = torch.where((g02 > g13).unsqueeze(1), quads[:, split1], quads[:, split2]).reshape(-1, 3)
        return vd, faces, L_dev, surf_edges
    vq = vd[quads]
    m02 = (vq[:, 0] + vq[:, 2]) / 2
    m13 = (vq[:, 1] + vq[:, 3]) / 2
    centre = (m02 * g02.unsqueeze(1) + m13 * g13.unsqueeze(1)) / ((g02 + g13) + 1e-8).unsqueeze(1)
    cidx = total + torch.arange(quads.shape[0])
    ring = quads[:, [0, 1, 1, 2, 2, 3, 3, 0]].reshape(-1, 4, 2)
    faces = torch.cat([ring, cidx.reshape(-1, 1, 1).expand(-1, 4, 1)], -1).reshape(-1, 3)
    return torch.cat([vd, centre]), faces, L_dev, surf_edges
