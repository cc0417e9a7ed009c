"""A numpy model of the device algorithm on the dense on-grid layout (test infrastructure).

It executes, with numpy, the same arithmetic the CUDA kernels do on the same uploaded arrays: the 3-pass
FFT L_p product on this build's padded sizes, the stencil tail of the system product, the per-position
admittance blocks (with the positions' own blocks where strips are not full squares), the correction rows of
narrow strips and split layers' face couplings (narrow.cu), current sheets mapped to node layers (face
sheets), and the multifrontal LDL^T factorisation / triangular solves driven by the symbolic analysis.  Tests compare it with the oracle (so the arrays are right) and the GPU with it (so the kernels
are)."""
import numpy as np


class DenseModel:
    def __init__(self, st):
        self.st = st
        t, D = st.top, st.dense
        self.S, self.nx, self.ny = t.S, t.nx, t.ny
        self.NL = t.NL
        self.lay = np.asarray(t.sheet_layer, np.int64)     # each current sheet's node layer
        self.D = D
        self.np_ = len(t.pair_layers)
        # each capacitance cell's facing share (1 where whole or absent): its admittance is the pair's times it
        self.share = np.ones((self.np_, self.nx, self.ny))
        if t.cap_share is not None and len(t.cap_share):
            pidx = np.concatenate([np.full(int(t.cap_mask[p].sum()), p) for p in range(self.np_)])
            self.share[pidx, t.cap[:, 2].astype(int), t.cap[:, 3].astype(int)] = t.cap_share

    # ---------------------------------------------------------------- views
    def seg(self, v, name):
        S, nx, ny, D = self.S, self.nx, self.ny, self.D
        if name == "X":
            return v[..., D.off_x: D.off_x + S * (nx - 1) * ny].reshape(v.shape[:-1] + (S, nx - 1, ny))
        if name == "Y":
            return v[..., D.off_y: D.off_y + S * nx * (ny - 1)].reshape(v.shape[:-1] + (S, nx, ny - 1))
        if name == "C":
            return v[..., D.off_c: D.off_c + self.np_ * nx * ny].reshape(v.shape[:-1] + (self.np_, nx, ny))
        if name == "B":
            return v[..., D.off_b: D.off_b + self.st.nbr]
        if name == "V":
            NL = self.NL
            return v[..., D.off_v: D.off_v + NL * nx * ny].reshape(v.shape[:-1] + (NL, nx, ny))

    def to_dense(self, x_compact):
        v = np.zeros(self.D.n, complex)
        v[self.D.compact_to_dense] = x_compact
        return v

    def to_compact(self, v):
        return v[self.D.compact_to_dense]

    # ---------------------------------------------------------------- L_p (3-pass FFT)
    def lp(self, Xg, orient):
        """(S, n0, n1) currents -> (S, n0, n1) L_p product, through the quadrant spectrum."""
        P0, P1 = self.st.P[orient]
        Kq = self.st.spectrum[orient]            # (Q1, Q0, S, S), scaled by 1/(P0 P1)
        S, n0, n1 = Xg.shape
        T = np.fft.fft(Xg, n=P1, axis=2)          # pass A: row FFTs
        F = np.fft.fft(T, n=P0, axis=1)           # pass B: column FFTs ...
        q0 = np.minimum(np.arange(P0), P0 - np.arange(P0))
        q1 = np.minimum(np.arange(P1), P1 - np.arange(P1))
        K = Kq[q1][:, q0]                         # (P1, P0, S, S)
        G = np.einsum("cpts,spc->tpc", K, F)      # ... spectrum multiply-add ...
        T2 = np.fft.ifft(G, axis=1)[:, :n0, :] * P0   # ... inverse column FFT (unscaled)
        Y = np.fft.ifft(T2, axis=2)[:, :, :n1] * P1    # pass C: inverse row FFTs (unscaled)
        return Y

    # ---------------------------------------------------------------- system product
    def matvec(self, v, w, zs, zcap, zbr):
        """zs: the sheets' impedances (S,) then the split layers' face couplings (n_twins,)."""
        st = self.st
        t = st.top
        zsh, zm = zs[: self.S], zs[self.S:]
        out = np.zeros_like(v)
        X, Y, C, B, Vn = (self.seg(v, n) for n in "XYCBV")
        oX, oY, oC, oB, oV = (self.seg(out, n) for n in "XYCBV")
        Vs = Vn[self.lay]                         # a sheet's strips end on its layer's nodes
        oX[:] = (zsh[:, None, None] * X + 1j * w * self.lp(X, "x") - (Vs[:, :-1, :] - Vs[:, 1:, :])) * t.xb
        oY[:] = (zsh[:, None, None] * Y + 1j * w * self.lp(Y, "y") - (Vs[:, :, :-1] - Vs[:, :, 1:])) * t.yb
        for p, (u, l) in enumerate(t.pair_layers):
            oC[p] = (zcap[p] / self.share[p] * C[p] - (Vn[u] - Vn[l])) * t.cap_mask[p]
        Vf = Vn.reshape(-1)
        for n, (a, b) in enumerate(self.branch_dense()):
            oB[n] = zbr[n] * B[n] - (Vf[a] - Vf[b])
        self.corrections(v, out, w, zsh, zm)
        oV[:] = self.kcl(v)
        return out

    def corrections(self, v, out, w, zsh, zm):
        """The rows of strips that are not full squares and of face pairs (narrow.cu's system-product mode):
        out[p] += z (1/w_p - 1) x[p] + j omega (dL_p x[p] + sum_q M[p,q] x[q]) (+ the real part's factor)
        (+ the face coupling z_mut / width x[partner])."""
        nr = getattr(self.st, "narrow_rows", None)
        if nr is None:
            return
        for q in range(len(nr["pos"])):
            p, s = nr["pos"][q], nr["sheet"][q]
            lo, hi = nr["ptr"][q], nr["ptr"][q + 1]
            acc = nr["dl"][q] * v[p] + np.dot(nr["val"][lo:hi], v[nr["col"][lo:hi]])
            y = nr["rdelta"][q] * zsh[s] * v[p] + 1j * w * acc + nr["rre"][q] * zsh[s].real * v[p]
            if nr["partner"][q] >= 0:
                zq = zm[nr["twin"][q]]
                y += (nr["tw_fac"][q] * zq + nr["twre"][q] * zq.real) * v[nr["partner"][q]]
            out[p] += y

    def vmask(self):
        m = np.zeros(self.NL * self.nx * self.ny, bool)
        node_dense = np.flatnonzero(self.st.top.node.ravel())
        m[node_dense[self.st.top.keep]] = True
        return m.reshape(self.NL, self.nx, self.ny)

    def branch_dense(self):
        node_dense = np.flatnonzero(self.st.top.node.ravel())
        return node_dense[self.st.top.branch_ab]

    # ---------------------------------------------------------------- preconditioner
    def dinv(self, v, tab):
        """Apply D^-1 to the branch segments of v (per-position code tables, caps, branches)."""
        st = self.st
        S, ncode = self.S, 1 << self.S
        out = np.zeros_like(v)
        for o, name in ((0, "X"), (1, "Y")):
            A = self.seg(v, name)
            O = self.seg(out, name)
            code = st.code["x" if o == 0 else "y"].astype(np.int64)
            T = tab[: 2 * ncode * S * S].reshape(2, ncode, S, S)[o][code]      # (n0, n1, S, S)
            own = st.override["x" if o == 0 else "y"] if st.n_override else None
            if own is not None and (own >= 0).any():
                # a position whose strips are not all full squares: its own block, over the sheets present
                blocks = tab[st.tab_ovr0: st.tab_ovr0 + st.n_override * S * S].reshape(-1, S, S)
                sel = own >= 0
                bits = (code[sel][:, None] >> np.arange(S)[None, :]) & 1
                T[sel] = blocks[own[sel]] * (bits[:, :, None] * bits[:, None, :])
            O[:] = np.einsum("ijkl,lij->kij", T, A)
        C, oC = self.seg(v, "C"), self.seg(out, "C")
        for p in range(self.np_):
            oC[p] = tab[st.tab_cap0 + p] * self.share[p] * C[p] * st.top.cap_mask[p]
        self.seg(out, "B")[:] = tab[st.tab_br0: st.tab_br0 + st.nbr] * self.seg(v, "B")
        return out

    def kcl(self, v):
        """Ar^T applied to the branch segments: the node rows (masked by the kept nodes)."""
        t = self.st.top
        X, Y, C, B = (self.seg(v, n) for n in "XYCB")
        k = np.zeros((self.NL, self.nx, self.ny), complex)
        for s, L in enumerate(self.lay):          # a face sheet's strips join its layer's nodes
            k[L, :-1, :] += X[s]
            k[L, 1:, :] -= X[s]
            k[L, :, :-1] += Y[s]
            k[L, :, 1:] -= Y[s]
        for p, (u, l) in enumerate(t.pair_layers):
            k[u] += C[p]
            k[l] -= C[p]
        kf = k.reshape(-1)
        for n, (a, b) in enumerate(self.branch_dense()):
            kf[a] += B[n]
            kf[b] -= B[n]
        return k * self.vmask()

    def grad(self, Vn):
        """Ar applied to node potentials: per-branch-segment differences V[a] - V[b] (dense, unmasked)."""
        out = np.zeros(self.D.n, complex)
        Vs = Vn[self.lay]
        self.seg(out, "X")[:] = Vs[:, :-1, :] - Vs[:, 1:, :]
        self.seg(out, "Y")[:] = Vs[:, :, :-1] - Vs[:, :, 1:]
        C = self.seg(out, "C")
        for p, (u, l) in enumerate(self.st.top.pair_layers):
            C[p] = Vn[u] - Vn[l]
        Vf = Vn.reshape(-1)
        B = self.seg(out, "B")
        for n, (a, b) in enumerate(self.branch_dense()):
            B[n] = Vf[a] - Vf[b]
        return out

    def precond(self, v, tab, fac):
        sym = self.st.sym
        t1 = self.dinv(v, tab)
        s = self.seg(v, "V") - self.kcl(t1)
        s_fac = s.reshape(-1)[sym.iperm]
        y_fac = fac.solve(s_fac)
        yv = np.zeros(self.NL * self.nx * self.ny, complex)
        yv[sym.iperm] = y_fac
        yv = yv.reshape(self.NL, self.nx, self.ny)
        u = v + self.grad(yv)
        out = self.dinv(u, tab)
        out *= self.D.mask
        self.seg(out, "V")[:] = yv
        return out


class Multifrontal:
    """LDL^T of S by the symbolic analysis's fronts (what the device factorisation kernels do)."""

    def __init__(self, st, s_values):
        sym = st.sym
        self.sym = sym
        nfront = len(sym.nown)
        self.panels = [None] * nfront
        upd = [None] * nfront
        for h in range(len(sym.level_ptr) - 1):
            for f in sym.order[sym.level_ptr[h]: sym.level_ptr[h + 1]]:
                no, nbd = sym.nown[f], sym.nbnd[f]
                nf = no + nbd
                F = np.zeros((nf, nf), complex)
                e = slice(sym.ent_ptr[f], sym.ent_ptr[f + 1])
                np.add.at(F, (sym.ent_row[e], sym.ent_col[e]), s_values[sym.ent_s[e]])
                for ci in range(sym.child_ptr[f], sym.child_ptr[f + 1]):
                    c = sym.child_idx[ci]
                    m = sym.cmap_idx[sym.cmap_ptr[ci]: sym.cmap_ptr[ci + 1]]
                    F[np.ix_(m, m)] += upd[c]
                    upd[c] = None
                # F holds the lower triangle (assembly) plus update blocks (full): symmetrise from the lower
                F = np.tril(F) + np.tril(F, -1).T
                for k in range(no):
                    dk = F[k, k]
                    l = F[k + 1:, k] / dk
                    F[k + 1:, k + 1:] -= np.outer(l, l) * dk
                    F[k + 1:, k] = l
                self.panels[f] = F[:, :no].copy()
                upd[f] = F[no:, no:].copy()

    def solve(self, b):
        sym = self.sym
        z = b.astype(complex).copy()
        nlev = len(sym.level_ptr) - 1
        for h in range(nlev):
            for f in sym.order[sym.level_ptr[h]: sym.level_ptr[h + 1]]:
                o0, no = sym.own_start[f], sym.nown[f]
                Lp = self.panels[f]
                bnd = sym.bnd_idx[sym.bnd_ptr[f]: sym.bnd_ptr[f + 1]]
                for k in range(no):
                    z[o0 + k + 1: o0 + no] -= Lp[k + 1: no, k] * z[o0 + k]
                    z[bnd] -= Lp[no:, k] * z[o0 + k]
        for f in range(len(sym.nown)):
            o0, no = sym.own_start[f], sym.nown[f]
            z[o0: o0 + no] /= np.diag(self.panels[f][:no, :no])
        for h in range(nlev - 1, -1, -1):
            for f in sym.order[sym.level_ptr[h]: sym.level_ptr[h + 1]]:
                o0, no = sym.own_start[f], sym.nown[f]
                Lp = self.panels[f]
                bnd = sym.bnd_idx[sym.bnd_ptr[f]: sym.bnd_ptr[f + 1]]
                for k in range(no - 1, -1, -1):
                    z[o0 + k] -= Lp[no:, k] @ z[bnd] + Lp[k + 1: no, k] @ z[o0 + k + 1: o0 + no]
        return z


class LowRank:
    """A derived stack's factor (woodbury.cu, gt_operators_derive): the base's factorisation of S plus the added
    branches' update S' = S + U diag(1/z) U^T, solved as y - W (Z + U^T W)^-1 U^T y with y = S^-1 v and
    W = S^-1 U (U: per added branch +1 / -1 at its kept end nodes, in factor order)."""

    def __init__(self, model: DenseModel, fac, zbr):
        st = model.st
        sym = st.sym
        n0 = st.nbr - st.n_lowrank
        ends = model.branch_dense()[n0:]
        kept = model.vmask().reshape(-1)
        self.U = np.zeros((sym.n, st.n_lowrank))
        for k, (a, b) in enumerate(ends):
            if kept[a]:
                self.U[sym.perm[a], k] += 1.0
            if kept[b]:
                self.U[sym.perm[b], k] -= 1.0
        self.fac = fac
        self.W = np.stack([fac.solve(self.U[:, k].astype(complex)) for k in range(st.n_lowrank)], axis=1)
        self.Minv = np.linalg.inv(np.diag(zbr[n0:]) + self.U.T @ self.W)

    def solve(self, v):
        y = self.fac.solve(v)
        return y - self.W @ (self.Minv @ (self.U.T @ y))
