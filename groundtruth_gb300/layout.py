"""Index work of the plane solve, done once per geometry on the host.

1. The reference's unknown numbering (src/groundtruth/solver/peec.py:1596-1656, 1845-1862), bit-exact:
   node ids in np.nonzero order, x/y strips in np.argwhere order (sheet, i, j), plane-pair capacitances per
   pair in np.nonzero order, branches, incidence ends, connected components (conductive and full), one
   reference node per full component (its lowest node id) dropped from the potentials.

2. The device's *dense on-grid layout* of an unknown vector.  Every segment is a full grid with a mask:

       X  (S, nx-1, ny)  x-strip currents         Y  (S, nx, ny-1)  y-strip currents
       C  (npairs, nx, ny) capacitance currents   B  (nbr,)          branch currents
       V  (S, nx, ny)    node potentials (zero at reference and non-copper nodes)

   so the incidence products Ar V and Ar^T I are 5-point stencils instead of sparse products, and the FFT
   passes read and write whole grid rows.  Masked entries are kept exactly zero by every kernel.

3. The nested-dissection symbolic analysis of the Schur complement S = Ar^T D^-1 Ar on the kept nodes:
   geometric bisection of the (i, j) box by lines of positions (all layers of a position together),
   separators ordered after their two halves, branch ends that join distant boxes promoted to the lowest
   common separator; then the multifrontal structure (fronts, update-matrix maps, assembly lists) and the
   S-term matrix that assembles S from a small per-frequency admittance table on the device.
"""
from __future__ import annotations

from dataclasses import dataclass, replace

import numpy as np
import scipy.sparse as sp
from scipy.sparse.csgraph import connected_components

ALIGN = 64          # segment starts in the dense vector, in complex elements (512 B at FP32)


def _align(n: int) -> int:
    return (n + ALIGN - 1) // ALIGN * ALIGN


@dataclass
class Topology:
    S: int                    # current sheets (the layers, then the lower faces of split layers)
    nx: int
    ny: int
    node: np.ndarray          # (NL, nx, ny) bool, per layer
    xb: np.ndarray            # (S, nx-1, ny) bool (strip and both end nodes), per sheet
    yb: np.ndarray
    nid: np.ndarray           # (NL, nx, ny) int64, -1 off copper
    xa: np.ndarray            # (nxb, 3)
    ya: np.ndarray
    cap: np.ndarray           # (ncap, 6): upper, lower, i, j, C, tan_delta
    pair_layers: np.ndarray   # (npairs, 2)
    cap_mask: np.ndarray      # (npairs, nx, ny) bool
    branch_ab: np.ndarray     # (nbr, 2) node ids a, b
    a_nodes: np.ndarray
    b_nodes: np.ndarray
    cond_label: np.ndarray
    full_label: np.ndarray
    keep: np.ndarray          # (n_nodes,) bool
    sheet_layer: np.ndarray = None   # (S,) each sheet's layer (its strips join that layer's nodes)
    cap_share: np.ndarray = None     # (ncap,) each capacitance cell's facing copper share (1: whole cells)

    @property
    def NL(self):
        return self.node.shape[0]

    @property
    def n_nodes(self):
        return len(self.keep)

    @property
    def nxb(self):
        return len(self.xa)

    @property
    def ns(self):
        return len(self.xa) + len(self.ya)

    @property
    def ncap(self):
        return len(self.cap)

    @property
    def nbr(self):
        return len(self.branch_ab)

    @property
    def nb(self):
        return self.ns + self.ncap + self.nbr

    @property
    def n_keep(self):
        return int(self.keep.sum())


def topology(node_masks, xb_masks, yb_masks, d: float, pairs: list, branch_nodes: list, twin_parent=(),
             fills=None) -> tuple:
    """The reference's numbering (peec.py:1596-1656).  pairs: [(upper, lower, c_per_area, tan_delta)];
    branch_nodes: [((k,i,j), (k,i,j))]; twin_parent: the split layers, whose lower-face sheets (numbered after the
    layers) have the layer's strips on the layer's nodes; fills: per layer the cells' copper fraction (None, or
    None for a layer: its node mask), a plane pair's cell capacitance taking the smaller of its two layers'
    (peec.py:1622-1637).  Returns (Topology, indices of the branches kept: both ends on copper and different)."""
    node = np.stack(node_masks).astype(bool)
    NL, nx, ny = node.shape
    twin_parent = np.asarray(twin_parent, np.int64)
    xb = np.stack(xb_masks).astype(bool) & node[:, :-1, :] & node[:, 1:, :]
    yb = np.stack(yb_masks).astype(bool) & node[:, :, :-1] & node[:, :, 1:]
    if len(twin_parent):
        xb = np.concatenate([xb, xb[twin_parent]])
        yb = np.concatenate([yb, yb[twin_parent]])
    sheet_layer = np.concatenate([np.arange(NL), twin_parent]).astype(np.int64)
    S = NL + len(twin_parent)
    nid = -np.ones(node.shape, np.int64)
    idx = np.nonzero(node)
    nid[idx] = np.arange(len(idx[0]))
    n = len(idx[0])
    xa, ya = np.argwhere(xb), np.argwhere(yb)
    fill = [node[k].astype(float) if fills is None or fills[k] is None else np.asarray(fills[k], float)
            for k in range(NL)]
    caps, pl, cmask, shares = [], [], [], []
    for (u, l, cpa, td) in pairs:
        between = np.zeros((nx, ny), bool)
        for m in range(int(u) + 1, int(l)):
            between |= node[m]
        full = np.minimum(fill[int(u)], fill[int(l)])
        mask = node[int(u)] & node[int(l)] & ~between & (full > 0)
        ii, jj = np.nonzero(mask)
        share = full[ii, jj]
        caps.append(np.column_stack([np.full(len(ii), u), np.full(len(ii), l), ii, jj,
                                     cpa * (d * d) * share, np.full(len(ii), td)]))
        pl.append((int(u), int(l)))
        cmask.append(mask)
        shares.append(share)
    cap = np.concatenate(caps) if caps else np.zeros((0, 6))
    kept, ab = [], []
    for n_br, (a, b) in enumerate(branch_nodes):
        na, nbb = int(nid[tuple(a)]), int(nid[tuple(b)])
        if na >= 0 and nbb >= 0 and tuple(a) != tuple(b):
            kept.append(n_br)
            ab.append((na, nbb))
    ab = np.array(ab, np.int64).reshape(-1, 2)
    cu = cap[:, :4].astype(np.int64)
    lx, ly = sheet_layer[xa[:, 0]], sheet_layer[ya[:, 0]]          # a strip joins its layer's nodes
    a_nodes = np.concatenate([nid[lx, xa[:, 1], xa[:, 2]], nid[ly, ya[:, 1], ya[:, 2]],
                              nid[cu[:, 0], cu[:, 2], cu[:, 3]], ab[:, 0]]).astype(np.int64)
    b_nodes = np.concatenate([nid[lx, xa[:, 1] + 1, xa[:, 2]], nid[ly, ya[:, 1], ya[:, 2] + 1],
                              nid[cu[:, 1], cu[:, 2], cu[:, 3]], ab[:, 1]]).astype(np.int64)
    ns = len(xa) + len(ya)
    cond = np.ones(len(a_nodes), bool)
    cond[ns: ns + len(cap)] = False
    g = sp.coo_matrix((np.ones(cond.sum()), (a_nodes[cond], b_nodes[cond])), shape=(n, n))
    _, cond_label = connected_components(g, directed=False)
    g = sp.coo_matrix((np.ones(len(a_nodes)), (a_nodes, b_nodes)), shape=(n, n))
    _, full_label = connected_components(g, directed=False)
    _, first = np.unique(full_label, return_index=True)
    keep = np.ones(n, bool)
    keep[first] = False
    top = Topology(S, nx, ny, node, xb, yb, nid, xa, ya, cap, np.array(pl, np.int64).reshape(-1, 2),
                   np.array(cmask, bool).reshape(-1, nx, ny), ab, a_nodes, b_nodes, cond_label, full_label, keep,
                   sheet_layer, np.concatenate(shares) if shares else np.zeros(0))
    return top, kept


def add_branches(t: Topology, ab: np.ndarray) -> Topology:
    """t with more branches between node ids ab (k, 2) inside its pieces of copper (a derived stack,
    PlaneStack.with_branches, peec.py:1871-1912): the same strips, capacitances, nodes and reference nodes, the
    branches' ends appended to the incidence lists and the conductor components merged, numbered as topology()
    numbers them (connected_components: by each component's lowest node).  What topology() would give for the
    whole branch list, without redoing the grid's work."""
    ab = np.asarray(ab, np.int64).reshape(-1, 2)
    if np.any(t.full_label[ab[:, 0]] != t.full_label[ab[:, 1]]):
        raise ValueError("a branch joins two pieces of copper: the reference nodes change")
    nc = int(t.cond_label.max()) + 1 if len(t.cond_label) else 0
    g = sp.coo_matrix((np.ones(len(ab)), (t.cond_label[ab[:, 0]], t.cond_label[ab[:, 1]])), shape=(nc, nc))
    _, merged = connected_components(g, directed=False)
    lbl = merged[t.cond_label]
    _, first = np.unique(lbl, return_index=True)
    rank = np.empty(len(first), np.int64)
    rank[np.argsort(first)] = np.arange(len(first))
    return replace(t, branch_ab=np.concatenate([t.branch_ab, ab]),
                   a_nodes=np.concatenate([t.a_nodes, ab[:, 0]]), b_nodes=np.concatenate([t.b_nodes, ab[:, 1]]),
                   cond_label=rank[lbl].astype(t.cond_label.dtype))


@dataclass
class Dense:
    """Offsets (complex elements) of the segments of the dense vector and the reference <-> dense maps."""
    off_x: int
    off_y: int
    off_c: int
    off_b: int
    off_v: int
    n: int                  # total length
    compact_to_dense: np.ndarray   # (nb + n_keep,) dense position of each reference unknown
    mask: np.ndarray        # (n,) uint8: 1 where an unknown lives


def dense_layout(t: Topology) -> Dense:
    S, nx, ny = t.S, t.nx, t.ny
    nX, nY, nV = S * (nx - 1) * ny, S * nx * (ny - 1), t.NL * nx * ny
    nC = len(t.pair_layers) * nx * ny
    off_x = 0
    off_y = _align(off_x + nX)
    off_c = _align(off_y + nY)
    off_b = _align(off_c + nC)
    off_v = _align(off_b + t.nbr)
    n = _align(off_v + nV)
    xs = off_x + (t.xa[:, 0] * (nx - 1) + t.xa[:, 1]) * ny + t.xa[:, 2]
    ys = off_y + (t.ya[:, 0] * nx + t.ya[:, 1]) * (ny - 1) + t.ya[:, 2]
    # caps of pair p in np.nonzero order of its mask = the reference's per-pair order
    cs = []
    for p in range(len(t.pair_layers)):
        ii, jj = np.nonzero(t.cap_mask[p])
        cs.append(off_c + (p * nx + ii) * ny + jj)
    cs = np.concatenate(cs) if cs else np.zeros(0, np.int64)
    bs = off_b + np.arange(t.nbr)
    node_dense = np.flatnonzero(t.node.ravel())          # node id -> dense node index
    vs = off_v + node_dense[t.keep]
    c2d = np.concatenate([xs, ys, cs, bs, vs]).astype(np.int64)
    mask = np.zeros(n, np.uint8)
    mask[c2d] = 1
    return Dense(off_x, off_y, off_c, off_b, off_v, n, c2d, mask)


# ------------------------------------------------------------------------------------------ symbolic
def update_slots(height: np.ndarray, parent: np.ndarray, size: np.ndarray) -> tuple:
    """Element offsets of the fronts' update matrices, storage shared between matrices that are never live at
    the same time, and the storage's length.  The factorisation runs level by level (a front's level is its
    height in the elimination tree): front f's matrix is written at its own level and read when its parent's
    level assembles it, so it is live over levels height[f] .. height[parent[f]], both ends included (at a
    level, fronts read their children's matrices while other fronts of the level write theirs).  Slots are
    placed first fit over the free blocks, the largest matrices of a level first; a block comes free after the
    last level of its matrix."""
    import bisect
    nfront = len(size)
    end = np.where(parent >= 0, height[np.maximum(parent, 0)], height)
    nlev = int(height.max()) + 1 if nfront else 0
    starts = [[] for _ in range(nlev)]
    ends = [[] for _ in range(nlev)]
    for f in range(nfront):
        if size[f] > 0:
            starts[int(height[f])].append(f)
            ends[int(end[f])].append(f)
    off = np.zeros(nfront, np.int64)
    free_off, free_len = [], []          # free blocks below the high-water mark, sorted by offset, merged
    top = 0

    def release(o, n):
        i = bisect.bisect_left(free_off, o)
        if i > 0 and free_off[i - 1] + free_len[i - 1] == o:          # joins the block before it
            i -= 1
            free_len[i] += n
        else:
            free_off.insert(i, o)
            free_len.insert(i, n)
        if i + 1 < len(free_off) and free_off[i] + free_len[i] == free_off[i + 1]:   # and the one after it
            free_len[i] += free_len.pop(i + 1)
            free_off.pop(i + 1)

    for h in range(nlev):
        for f in sorted(starts[h], key=lambda f: -int(size[f])):
            n = int(size[f])
            for i in range(len(free_off)):
                if free_len[i] >= n:
                    off[f] = free_off[i]
                    if free_len[i] == n:
                        free_off.pop(i)
                        free_len.pop(i)
                    else:
                        free_off[i] += n
                        free_len[i] -= n
                    break
            else:
                if free_off and free_off[-1] + free_len[-1] == top:       # extend the last free block
                    off[f] = free_off.pop()
                    free_len.pop()
                else:
                    off[f] = top
                top = int(off[f]) + n
        for f in ends[h]:
            release(int(off[f]), int(size[f]))
    return off, top


@dataclass
class Symbolic:
    n: int                       # kept nodes (factor dimension)
    perm: np.ndarray             # dense node index -> factor index (-1: not kept)
    iperm: np.ndarray            # factor index -> dense node index
    own_start: np.ndarray        # per front: first factor index of its own (contiguous) nodes
    nown: np.ndarray
    nbnd: np.ndarray
    bnd_ptr: np.ndarray          # CSR of boundary factor indices
    bnd_idx: np.ndarray
    parent: np.ndarray
    height: np.ndarray
    order: np.ndarray            # fronts sorted by height
    level_ptr: np.ndarray        # order[level_ptr[h]:level_ptr[h+1]] have height h
    child_ptr: np.ndarray        # CSR of children
    child_idx: np.ndarray
    cmap_ptr: np.ndarray         # per child (in child_idx order): its bnd entries' positions in the parent front
    cmap_idx: np.ndarray
    panel_off: np.ndarray        # per front: element offset of its L panel (nf x nown, column-major)
    upd_off: np.ndarray          # per front: element offset of its update matrix (nbnd x nbnd, column-major)
    vec_off: np.ndarray          # per front: element offset of its update vector (nbnd) in a column's workspace
    panel_total: int
    upd_total: int
    vec_total: int
    ent_ptr: np.ndarray          # per front: CSR over its assembly entries
    ent_row: np.ndarray          # front row of each entry (int32)
    ent_col: np.ndarray          # front column (own) of each entry
    ent_s: np.ndarray            # index of the S value
    s_row: np.ndarray            # S lower-triangle entries (factor indices, row >= col)
    s_col: np.ndarray


def _nd_tree(pos_i, pos_j, nx, ny, leaf: int):
    """Geometric nested dissection on positions.  Returns (owner front per node, parent per front, box
    per front) with children numbered before parents (postorder)."""
    owner = np.full(len(pos_i), -1, np.int64)
    parent: list = []
    fronts_nodes: list = []

    # iterative post-order over boxes: stack of (i0, i1, j0, j1, node index array, parent slot, state)
    def build(i0, i1, j0, j1, nodes):
        """Returns the front id of this box's root (postorder numbering)."""
        if len(nodes) <= leaf or (i1 - i0 <= 1 and j1 - j0 <= 1):
            fid = len(parent)
            parent.append(-1)
            fronts_nodes.append(nodes)
            return fid
        if i1 - i0 >= j1 - j0:
            mid = (i0 + i1) // 2
            pi = pos_i[nodes]
            sep = nodes[pi == mid]
            lo, hi = nodes[pi < mid], nodes[pi > mid]
            kids = [build(i0, mid, j0, j1, lo) if len(lo) else None, build(mid + 1, i1, j0, j1, hi) if len(hi) else None]
        else:
            mid = (j0 + j1) // 2
            pj = pos_j[nodes]
            sep = nodes[pj == mid]
            lo, hi = nodes[pj < mid], nodes[pj > mid]
            kids = [build(i0, i1, j0, mid, lo) if len(lo) else None, build(i0, i1, mid + 1, j1, hi) if len(hi) else None]
        fid = len(parent)
        parent.append(-1)
        fronts_nodes.append(sep)
        for c in kids:
            if c is not None:
                parent[c] = fid
        return fid

    import sys
    old = sys.getrecursionlimit()
    sys.setrecursionlimit(max(old, 10000))
    try:
        build(0, nx, 0, ny, np.arange(len(pos_i)))
    finally:
        sys.setrecursionlimit(old)
    for f, nodes in enumerate(fronts_nodes):
        owner[nodes] = f
    return owner, np.array(parent, np.int64)


def _ancestors(parent):
    """depth per front (root depth 0)."""
    nf = len(parent)
    depth = np.zeros(nf, np.int64)
    for f in range(nf - 1, -1, -1):          # parents have larger ids (postorder)
        if parent[f] >= 0:
            depth[f] = depth[parent[f]] + 1
    return depth


def _lca(a: np.ndarray, b: np.ndarray, parent: np.ndarray, depth: np.ndarray) -> np.ndarray:
    """The lowest common ancestor of fronts a[q] and b[q], for all q at once: the deeper one lifted to the
    other's depth, then both together until they meet."""
    a, b = a.copy(), b.copy()
    for x, y in ((a, b), (b, a)):
        m = depth[x] > depth[y]
        while m.any():
            x[m] = parent[x[m]]
            m = depth[x] > depth[y]
    m = a != b
    while m.any():
        a[m], b[m] = parent[a[m]], parent[b[m]]
        m = a != b
    return a


def symbolic(t: Topology, S_pattern: sp.csr_matrix, leaf: int = 48) -> Symbolic:
    """Nested-dissection multifrontal analysis of S (pattern on kept nodes in reference order)."""
    node_dense = np.flatnonzero(t.node.ravel())
    kept_dense = node_dense[t.keep]                      # reference kept order -> dense node index
    nxy = t.nx * t.ny
    pos = kept_dense % nxy
    pos_i, pos_j = pos // t.ny, pos % t.ny
    owner, parent = _nd_tree(pos_i, pos_j, t.nx, t.ny, leaf)
    depth = _ancestors(parent)
    # promote the ends of edges that join unrelated fronts (long-range branches) to their lowest common
    # ancestor until every edge joins a front and one of its ancestors or descendants
    coo = sp.triu(S_pattern, k=1).tocoo()
    u, v = coo.row, coo.col
    while True:
        fu, fv = owner[u], owner[v]
        diff = fu != fv
        a, b, fa, fb = u[diff], v[diff], fu[diff], fv[diff]
        l = _lca(fa, fb, parent, depth)
        bad = (l != fa) & (l != fb)
        if not bad.any():
            break
        # both ends of each such edge move to the ancestor, the edges taken in order (a node on several takes
        # the last one's)
        ends = np.stack([a[bad], b[bad]], axis=1).ravel()[::-1]
        to = np.repeat(l[bad], 2)[::-1]
        nodes, last = np.unique(ends, return_index=True)
        owner[nodes] = to[last]
    nfront = len(parent)
    # factor order: fronts in postorder, within a front by (i, j, layer)
    key = np.lexsort((kept_dense // nxy, pos_j, pos_i, owner))
    n = len(key)
    fac_of_kept = np.empty(n, np.int64)
    fac_of_kept[key] = np.arange(n)
    perm = -np.ones(t.NL * nxy, np.int64)
    perm[kept_dense] = fac_of_kept
    iperm = kept_dense[key]
    counts = np.bincount(owner, minlength=nfront)
    own_start = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    # pattern in factor order, lower triangle
    P = S_pattern.tocoo()
    fr, fc = fac_of_kept[P.row], fac_of_kept[P.col]
    lower = fr >= fc
    s_row, s_col = fr[lower], fc[lower]
    o = np.lexsort((s_row, s_col))
    s_row, s_col = s_row[o], s_col[o]
    front_of_fac = np.repeat(np.arange(nfront), counts)
    # boundaries (multifrontal symbolic): own adjacency beyond the own block, plus children's boundaries
    children = [[] for _ in range(nfront)]
    for f in range(nfront):
        if parent[f] >= 0:
            children[parent[f]].append(f)
    col_ptr = np.searchsorted(s_col, np.arange(n + 1))
    bnd = [None] * nfront
    for f in range(nfront):
        lo, hi = own_start[f], own_start[f] + counts[f]
        rows = s_row[col_ptr[lo]: col_ptr[hi]]
        parts = [rows[rows >= hi]] + [bnd[c][bnd[c] >= hi] for c in children[f]]
        bnd[f] = np.unique(np.concatenate(parts)) if parts else np.zeros(0, np.int64)
    nbnd = np.array([len(b) for b in bnd], np.int64)
    nown = counts.astype(np.int64)
    nf = nown + nbnd
    bnd_ptr = np.concatenate([[0], np.cumsum(nbnd)]).astype(np.int64)
    bnd_idx = np.concatenate(bnd).astype(np.int64) if nfront else np.zeros(0, np.int64)
    # heights and levels
    height = np.zeros(nfront, np.int64)
    for f in range(nfront):
        if parent[f] >= 0:
            height[parent[f]] = max(height[parent[f]], height[f] + 1)
    order = np.argsort(height, kind="stable")
    level_ptr = np.searchsorted(height[order], np.arange(height.max() + 2))
    child_ptr = np.concatenate([[0], np.cumsum([len(c) for c in children])]).astype(np.int64)
    child_idx = np.array([c for cs in children for c in cs], np.int64)
    cmaps = []
    for f in range(nfront):
        struct = np.concatenate([np.arange(own_start[f], own_start[f] + nown[f]), bnd[f]])
        for c in children[f]:
            # own indices ascending, then bnd ascending, all own < all bnd: struct is sorted
            m = np.searchsorted(struct, bnd[c])
            if len(m) and (m.max() >= len(struct) or not np.array_equal(struct[m], bnd[c])):
                raise AssertionError("symbolic: a child's boundary is not inside its parent's front")
            cmaps.append(m)
    cmap_ptr = np.concatenate([[0], np.cumsum([len(m) for m in cmaps])]).astype(np.int64)
    cmap_idx = np.concatenate(cmaps).astype(np.int64) if cmaps else np.zeros(0, np.int64)
    panel = nf * nown
    panel_off = np.concatenate([[0], np.cumsum(panel)[:-1]]).astype(np.int64)
    upd = nbnd * nbnd
    upd_off, upd_total = update_slots(height, parent, upd)
    vec_off = np.concatenate([[0], np.cumsum(nbnd)[:-1]]).astype(np.int64)
    # assembly entries: S lower entry (r, c) goes to the front owning column c
    ef = front_of_fac[s_col]
    ecol = s_col - own_start[ef]
    erow = np.empty(len(s_row), np.int64)
    in_own = s_row < own_start[ef] + nown[ef]
    erow[in_own] = s_row[in_own] - own_start[ef[in_own]]
    # boundary rows: the entries below each front's own block, grouped by front (one sort, no per-front scan)
    oi = np.flatnonzero(~in_own)
    of = ef[oi]
    so = np.argsort(of, kind="stable")
    oi, of = oi[so], of[so]
    cut = np.flatnonzero(np.diff(of)) + 1
    for s0, s1 in zip(np.concatenate([[0], cut]), np.concatenate([cut, [len(oi)]])):
        if s1 <= s0:
            continue
        f = of[s0]
        sel = oi[s0:s1]
        pos = np.searchsorted(bnd[f], s_row[sel])
        if np.any(pos >= nbnd[f]) or not np.array_equal(bnd[f][pos], s_row[sel]):
            raise AssertionError("symbolic: an entry of S is not on its front's boundary")
        erow[sel] = nown[f] + pos
    nfe = (nown + nbnd)[ef]
    if len(erow) and (erow.min() < 0 or np.any(erow >= nfe) or np.any(erow < ecol)):
        raise AssertionError("symbolic: an entry of S falls outside its front")
    eo = np.argsort(ef, kind="stable")
    ent_ptr = np.searchsorted(ef[eo], np.arange(nfront + 1)).astype(np.int64)
    return Symbolic(n, perm, iperm, own_start, nown, nbnd, bnd_ptr, bnd_idx, parent, height, order.astype(np.int64),
                    level_ptr.astype(np.int64), child_ptr, child_idx, cmap_ptr, cmap_idx, panel_off, upd_off, vec_off,
                    int(panel.sum()), upd_total, int(nbnd.sum()), ent_ptr, erow[eo], ecol[eo], eo.astype(np.int64),
                    s_row, s_col)
