"""CPU restatement of KAPDQMC's projector-DQMC sweep (``phy_update``).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, the smoke check and the CPU
baseline leg of the benchmark as the checker; the product never calls it.

It follows the reference operation by operation and keeps its LAPACK routine
choices (``?gerqf/?orgrq`` for the left chain, ``?geqrf/?orgqr`` for the
right chain, ``?getrf/?getrs`` for the Green's-function recompute), taking
the random stream from an explicit proposal tape (``k``, ``u``) in the
reference's consumption order instead of an unseedable MersenneTwister.

Parity is unpinned: the reference is Julia (not installed here) and ships no
golden vectors; this restatement is checked by invariants instead (the
brute-force ``Gτ`` recompute, free-fermion energies, eK*eKinv = I) and by
known answers that share none of its arithmetic: on 8-site lattices its
chains reproduce the exact Fock-space sums of the same weights
(fock_oracle.py; energies, structure factors, Rényi-2 and disorder ratios),
and those sums converge to exact diagonalisation of the Hamiltonians.

References (KAPDQMC): src/tU/phy_update.jl, src/tU/GreenMatrix.jl,
src/tV/phy_update.jl, src/tV/GreenMatrix.jl, src/tUV/phy_update.jl,
src/tUV/GreenMatrix.jl, src/public/Gupdate.jl, src/public/GF.jl.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.linalg import lapack

KIND_TU, KIND_TV, KIND_TUV = 0, 1, 2


class Tape:
    """Sequential proposal tape: ``k`` in {0,1,2} and ``u`` in [0,1)."""

    def __init__(self, k, u):
        self.k = np.asarray(k, dtype=np.uint8)
        self.u = np.asarray(u, dtype=np.float64)
        self.pos = 0

    def draw(self):
        if self.pos >= len(self.k):
            raise IndexError("proposal tape exhausted")
        k, u = int(self.k[self.pos]), float(self.u[self.pos])
        self.pos += 1
        return k, u


def _sx(sold: int, k: int) -> int:
    """k-th element of {1,2,3,4} minus sold (ascending): src/tU/model.jl:87-93."""
    return (1, 2, 3, 4, 5)[k + (k + 1 >= sold)]


# --------------------------------------------------------------------------
# shared numerics: src/public/Gupdate.jl
# --------------------------------------------------------------------------
def _lp(dtype):
    c = np.issubdtype(dtype, np.complexfloating)
    return (lapack.zgerqf if c else lapack.dgerqf, lapack.zungrq if c else lapack.dorgrq,
            lapack.zgeqrf if c else lapack.dgeqrf, lapack.zungqr if c else lapack.dorgqr,
            lapack.zgetrf if c else lapack.dgetrf, lapack.zgetrs if c else lapack.dgetrs)


def orth_rows(A):
    """Orthonormal rows spanning A's row space: gerqf! + orgrq! (src/tU/phy_update.jl:43-46)."""
    gerqf, orgrq, *_ = _lp(A.dtype)
    rq, tau, _, info = gerqf(A)
    assert info == 0
    q, _, info = orgrq(rq, tau)
    assert info == 0
    return q


def orth_cols(A):
    """Orthonormal columns spanning A's column space: geqrf! + orgqr! (src/tU/phy_update.jl:84-87)."""
    _, _, geqrf, orgqr, _, _ = _lp(A.dtype)
    qr, tau, _, info = geqrf(A)
    assert info == 0
    q, _, info = orgqr(qr, tau)
    assert info == 0
    return q


def get_G(BL, BR):
    """G = I - BR (BL BR)^-1 BL via getrf + getrs.  src/public/Gupdate.jl:139-157."""
    *_, getrf, getrs = _lp(BL.dtype)
    lu, piv, info = getrf(BL @ BR)
    assert info == 0, "singular BL*BR"
    X, info = getrs(lu, piv, BL)
    assert info == 0
    G = -(BR @ X)
    G[np.diag_indices_from(G)] += 1
    return G


def Gupdate(G, S, r):
    """G -= G[:,S] r (E_S - G[S,:]).  src/public/Gupdate.jl:5-11."""
    zN = -(r @ G[S, :])
    zN[:, S] += r
    G -= G[:, S] @ zN


def inv22(B):
    """2x2 inverse by the adjugate.  src/public/GF.jl:75-81."""
    d = B[0, 0] * B[1, 1] - B[0, 1] * B[1, 0]
    return np.array([[B[1, 1], -B[0, 1]], [-B[1, 0], B[0, 0]]]) / d


def det22(B):
    return B[0, 0] * B[1, 1] - B[0, 1] * B[1, 0]


# --------------------------------------------------------------------------
# model-specific slice matrices
# --------------------------------------------------------------------------
class _Sweep:
    """Common sweep driver state (PhyBuffer_, src/public/Buffer.jl:3-19)."""

    def __init__(self, model, s, tape: Tape, record: bool):
        self.m = model
        self.s = np.array(s, dtype=np.uint8, order="F", copy=True)
        self.tape = tape
        self.record = record
        self.NN = len(model.nodes)
        self.Θidx = self.NN // 2 + 1
        self.nodes = [int(v) for v in model.nodes]
        self.node_set = set(self.nodes)
        self.accepts: list = []
        self.drift: list = []
        self.obs_rows: list = []
        self.sweep_no = 0          # Philox sweep counter of the cluster moves
        self.slmc = None           # cluster-move configuration (t-U), see phy_update
        self.slmc_log: list = []   # (u, p) of every cluster-move decision
        self.full_sf = False       # t-U, complex t-UV: append the structure factors with all terms

    def node(self, k):  # 1-based access to nodes
        return self.nodes[k - 1]

    # forward/backward stabilisation --------------------------------------
    def init_chain(self):
        m, NN = self.m, self.NN
        self.BRs = [None] * (NN + 1)
        self.BLs = [None] * (NN + 1)
        self.BRs[1] = m.Pt.astype(self.dtype)
        self.BLs[NN] = m.Pt.conj().T.astype(self.dtype)
        for idx in range(NN - 1, 0, -1):
            self.BLs[idx] = orth_rows(self.BLs[idx + 1] @ self.BM(idx))
        self.idx = 1
        self.G = get_G(self.BLs[1], self.BRs[1])

    def _recompute(self):
        G_new = get_G(self.BLs[self.idx], self.BRs[self.idx])
        nrm = np.linalg.norm(G_new)
        self.drift.append(float(np.linalg.norm(self.G - G_new) / nrm))
        self.G = G_new

    def node_forward(self):
        self.idx += 1
        self.BRs[self.idx] = orth_cols(self.BM(self.idx - 1) @ self.BRs[self.idx - 1])
        self._recompute()

    def node_backward(self):
        self.idx -= 1
        self.BLs[self.idx] = orth_rows(self.BLs[self.idx + 1] @ self.BM(self.idx))
        self._recompute()

    def BM(self, idx):
        """Block product of slices node(idx)+1 .. node(idx+1) (BM_F!)."""
        M = np.eye(self.m.Ns, dtype=self.dtype)
        for lt in range(self.node(idx) + 1, self.node(idx + 1) + 1):
            M = self.B_left(lt, M)
        return M


class _TUSweep(_Sweep):
    """t-U model.  src/tU/phy_update.jl:3-267, src/tU/GreenMatrix.jl:10-86."""
    dtype = np.complex128

    def D(self, lt, sign=1.0):
        m = self.m
        return np.exp(1j * sign * m.α[lt - 1] * m.η[self.s[:, lt - 1].astype(np.int64) - 1])

    def B_left(self, lt, M):  # D(lt) eK M   (BM_F!, GreenMatrix.jl:20-26)
        return self.D(lt)[:, None] * (self.m.eK @ M)

    def wrap_forward(self, G, lt):  # WrapKV!("Forward","B"), GreenMatrix.jl:64-69
        d = self.D(lt)
        G = self.m.eK @ G @ self.m.eKinv
        return d[:, None] * G * (1.0 / d)[None, :]

    def wrap_backward(self, G, lt):  # WrapKV!("Backward","B"), GreenMatrix.jl:78-83
        d = self.D(lt, -1.0)
        G = d[:, None] * G * (1.0 / d)[None, :]
        return self.m.eKinv @ G @ self.m.eK

    def update_layer(self, lt):  # UpdatePhyLayer!, phy_update.jl:256-267
        m, G, s = self.m, self.G, self.s
        for i in range(m.Ns):
            k, u = self.tape.draw()
            sold = int(s[i, lt - 1])
            sx = _sx(sold, k)
            Δ = np.exp(1j * m.α[lt - 1] * (m.η[sx - 1] - m.η[sold - 1])) - 1     # get_r!
            pc = 1 + Δ * (1 - G[i, i])
            r = Δ / pc
            p = (pc.real ** 2 + pc.imag ** 2) * m.γ[sx - 1] / m.γ[sold - 1]
            acc = u < p
            self.accepts.append(acc)
            if acc:
                Gupdate(G, [i], np.array([[r]]))
                s[i, lt - 1] = sx

    def after_update(self, lt, visit):
        if self.slmc is not None:
            self.slmc_moves(lt, visit)

    def slmc_moves(self, lt, visit):
        """Self-learning cluster moves at slice lt (no counterpart in the
        reference).  ``Lc`` consecutive sites from a random start, ``steps``
        Metropolis steps on exp(F) prod gamma with F the effective model
        (recomputed in full for every trial here), then the changed sites are
        accepted with |det(I + Delta_S (I - G_SS))|^2 exp(-(F' - F)) and G is
        updated by Gupdate! (src/public/Gupdate.jl:5-11) with
        r = (I + Delta_S (I - G_SS))^-1 Delta_S.  Random numbers: Philox4x32-10
        on (q, sweep, chain, 0x534C4D43) with q = (visit moves + move)(steps + 1) + step."""
        import cnn_oracle
        import philox

        cfg, m, G, s = self.slmc, self.m, self.G, self.s
        N, Lc, ne, t0 = m.Ns, cfg["cluster_len"], cfg["steps"], lt - 1
        key = (cfg["seed"] & 0xFFFFFFFF, cfg["seed"] >> 32)

        def draw(q):
            return [int(v) for v in philox.philox4x32_10(q & 0xFFFFFFFF, self.sweep_no & 0xFFFFFFFF,
                                                         cfg["chain"], 0x534C4D43, *key)]

        def u53(a, b):
            return ((a >> 5) * 67108864.0 + (b >> 6)) * (1.0 / 9007199254740992.0)

        for mv in range(cfg["moves"]):
            q0 = (visit * cfg["moves"] + mv) * (ne + 1)
            r = draw(q0)
            i0 = (r[0] * N) >> 32
            uf = u53(r[1], r[2])
            sites = [(i0 + k) % N for k in range(Lc)]
            orig = [int(s[j, t0]) for j in sites]
            cur = list(orig)
            field = np.ascontiguousarray(np.asarray(s, dtype=np.uint8).T)[None].copy()
            F = cnn_oracle.forward(field, cfg["params"])[0][0]
            dF_tot = 0.0
            for st in range(1, ne + 1):
                r = draw(q0 + st)
                k = (r[0] * Lc) >> 32
                kv = (r[1] * 3) >> 32
                u = u53(r[2], r[3])
                sold = cur[k]
                sx = _sx(sold, kv)
                trial = field.copy()
                trial[0, t0, sites[k]] = sx
                F1 = cnn_oracle.forward(trial, cfg["params"])[0][0]
                p = math.exp(F1 - F) * (m.γ[sx - 1] / m.γ[sold - 1])
                self.slmc_log.append((u, p))
                if u < p:
                    cur[k] = sx
                    field = trial
                    dF_tot += F1 - F
                    F = F1
            S = [k for k in range(Lc) if cur[k] != orig[k]]
            if not S:
                continue
            idx = [sites[k] for k in S]
            Δ = np.array([np.exp(1j * m.α[lt - 1] * (m.η[cur[k] - 1] - m.η[orig[k] - 1])) - 1 for k in S])
            M = np.eye(len(S)) + Δ[:, None] * (np.eye(len(S)) - G[np.ix_(idx, idx)])
            _, ld = np.linalg.slogdet(M)
            p = math.exp(2.0 * ld - dF_tot)
            self.slmc_log.append((uf, p))
            if uf < p:
                Gupdate(G, idx, np.linalg.inv(M) * Δ[None, :])
                for k in S:
                    s[sites[k], t0] = cur[k]

    def measure(self, lt):  # phy_measure, phy_update.jl:154-254
        m = self.m
        G0 = self.G.copy()
        half = m.Nt // 2
        if lt > m.Nt / 2:
            for t in range(lt, half, -1):
                G0 = self.wrap_backward(G0, t)
        else:
            for t in range(lt + 1, half + 1):
                G0 = self.wrap_forward(G0, t)
        G0 = m.HalfeK @ G0 @ m.HalfeKinv
        Ek = -2 * m.Ht * np.real(np.sum(m.K * G0))
        d = np.diag(G0)
        Eu = np.sum((1 - d) * d.conj())
        assert Eu.imag < 1e-8
        out = [Ek, Eu.real, 0.0, 0.0, 0.0, 0.0]
        if "HoneyComb" in m.Lattice:
            out[2:] = _honeycomb_sf_quirk(m.site, G0, m.Ns, spinful_real=False)
        if self.full_sf:
            out += _honeycomb_sf_full(m.site, G0, m.Ns) if "HoneyComb" in m.Lattice else _square_sf_full(m, G0)
        return np.array(out)

    def run(self, sweeps):
        m = self.m
        self.init_chain()
        for _ in range(sweeps):
            acc, cnt = np.zeros(10 if self.full_sf else 6), 0
            for lt in range(1, m.Nt + 1):
                self.G = self.wrap_forward(self.G, lt)
                self.update_layer(lt)
                self.after_update(lt, lt - 1)
                if self.record and 0 <= self.Θidx - self.idx <= 1:
                    acc += self.measure(lt)
                    cnt += 1
                if lt in self.node_set:
                    self.node_forward()
            for lt in range(m.Nt, 0, -1):
                self.update_layer(lt)
                self.after_update(lt, 2 * m.Nt - lt)
                if self.record and 0 <= self.idx - self.Θidx <= 1:
                    acc += self.measure(lt)
                    cnt += 1
                self.G = self.wrap_backward(self.G, lt)
                if lt - 1 in self.node_set:
                    self.node_backward()
            if self.record:
                self.obs_rows.append(acc / cnt)
            self.sweep_no += 1
        return self


class _TVSweep(_Sweep):
    """t-V model.  src/tV/phy_update.jl:1-314, src/tV/GreenMatrix.jl:12-119.

    The bond rotations UV_j are applied as the 2x2 blocks they are instead of
    dense GEMMs; the arithmetic per entry is the same two-term sum.
    """
    dtype = np.float64
    c = 2 ** 0.5 / 2
    uv = np.array([[-c, -c], [-c, c]])

    def __init__(self, *a, **k):
        super().__init__(*a, **k)
        nn = self.m.nnidx
        self.X = [nn[:, j, 0] - 1 for j in range(nn.shape[1])]   # A ends, 0-based
        self.Y = [nn[:, j, 1] - 1 for j in range(nn.shape[1])]   # B ends

    def Dj(self, lt, j, sign):
        """exp(±αη) on the A end, exp(∓αη) on the B end of each bond of direction j."""
        m = self.m
        v = m.α[lt - 1] * m.η[self.s[:, j, lt - 1].astype(np.int64) - 1]
        d = np.empty(m.Ns)
        d[self.X[j]] = v
        d[self.Y[j]] = -v
        return np.exp(sign * d)

    def uvL(self, j, G):  # UV_j @ G
        X, Y, c = self.X[j], self.Y[j], self.c
        out = np.empty_like(G)
        out[X] = -c * G[X] - c * G[Y]
        out[Y] = -c * G[X] + c * G[Y]
        return out

    def uvR(self, j, G):  # G @ UV_j
        return self.uvL(j, G.T).T

    def wrapV(self, G, j, d):  # WrapV!("B"), GreenMatrix.jl:110-118
        G = self.uvR(j, self.uvL(j, G))
        G = d[:, None] * G * (1.0 / d)[None, :]
        return self.uvR(j, self.uvL(j, G))

    def B_left(self, lt, M):  # BM_F!, GreenMatrix.jl:23-37
        M = self.m.eK @ M
        for j in reversed(range(self.m.z)):
            M = self.uvL(j, self.Dj(lt, j, 1.0)[:, None] * self.uvL(j, M))
        return M

    def update_layer(self, lt, j):  # UpdatePhyLayer!, phy_update.jl:190-205
        m, G, s, uv = self.m, self.G, self.s, self.uv
        for i in range(m.Ns // 2):
            x, y = int(self.X[j][i]), int(self.Y[j][i])
            S = [x, y]
            k, u = self.tape.draw()
            sold = int(s[i, j, lt - 1])
            sx = _sx(sold, k)
            Δs = m.α[lt - 1] * (m.η[sx - 1] - m.η[sold - 1])               # get_r!, GreenMatrix.jl:76-89
            t2 = np.exp(Δs * np.array([1.0, -1.0])) - 1
            Δ = (uv * t2[None, :]) @ uv
            r = Δ - Δ @ G[np.ix_(S, S)]
            r[0, 0] += 1
            r[1, 1] += 1
            p = det22(r)
            r = inv22(r) @ Δ
            p *= m.γ[sx - 1] / m.γ[sold - 1]
            acc = u < p
            self.accepts.append(acc)
            if acc:
                Gupdate(G, S, r)
                s[i, j, lt - 1] = sx

    def measure(self, lt):  # phy_measure, phy_update.jl:207-314 (xy_i called correctly)
        m = self.m
        G0 = self.G.copy()
        half = m.Nt // 2
        if lt > m.Nt / 2:
            for t in range(lt, half, -1):
                for j in range(m.z):
                    G0 = self.wrapV(G0, j, self.Dj(t, j, -1.0))
                G0 = m.eKinv @ G0 @ m.eK
        else:
            for t in range(lt + 1, half + 1):
                G0 = m.eK @ (G0 @ m.eKinv)
                for j in reversed(range(m.z)):
                    G0 = self.wrapV(G0, j, self.Dj(t, j, 1.0))
        G0 = m.HalfeK @ G0 @ m.HalfeKinv
        Ek = m.Ht * np.sum(m.K * G0)
        x = m.nnidx[:, :, 0].ravel(order="F") - 1
        y = m.nnidx[:, :, 1].ravel(order="F") - 1
        Ev = np.sum((1 - G0[x, x]) * (1 - G0[y, y]) - G0[x, y] * G0[y, x])
        R0, R1 = np.zeros(4), np.zeros(4)
        if "HoneyComb" in m.Lattice:
            R0, R1 = _tv_density_sf(m.site, G0, m.Ns)
        return np.concatenate([[Ek, Ev], R0, R1])

    def run(self, sweeps):
        m = self.m
        self.init_chain()
        for _ in range(sweeps):
            acc, cnt = np.zeros(10), 0
            for lt in range(1, m.Nt + 1):
                self.G = m.eK @ (self.G @ m.eKinv)
                for j in reversed(range(m.z)):
                    self.G = self.wrapV(self.G, j, self.Dj(lt, j, 1.0))
                    self.update_layer(lt, j)
                if self.record and abs(self.idx - self.Θidx) <= 1:
                    acc += self.measure(lt)
                    cnt += 1
                if lt in self.node_set:
                    self.node_forward()
            for lt in range(m.Nt, 0, -1):
                for j in range(m.z):
                    self.update_layer(lt, j)
                    self.G = self.wrapV(self.G, j, self.Dj(lt, j, -1.0))
                self.G = (m.eKinv @ self.G) @ m.eK
                if self.record and abs(self.idx - self.Θidx) <= 1:
                    acc += self.measure(lt - 1)
                    cnt += 1
                if lt - 1 in self.node_set:
                    self.node_backward()
            if self.record:
                self.obs_rows.append(acc / cnt)
        return self


class _TUVSweep(_Sweep):
    """t-U-V model.  src/tUV/phy_update.jl:1-355, src/tUV/GreenMatrix.jl:10-122."""

    def __init__(self, *a, **k):
        super().__init__(*a, **k)
        self.dtype = np.complex128 if self.m.is_complex else np.float64
        nn = self.m.nnidx
        self.X = nn[:, :, 0].ravel(order="F") - 1    # linear (column-major) bond order
        self.Y = nn[:, :, 1].ravel(order="F") - 1

    def phase(self, lt, sign):
        m = self.m
        e = m.η[self.s[:, lt - 1].astype(np.int64) - 1]
        v = np.zeros(m.Ns)
        np.add.at(v, self.X, e)
        np.add.at(v, self.Y, m.a * e)
        return np.exp(1j * sign * v) if m.is_complex else np.exp(sign * v)

    def B_left(self, lt, M):  # BM_F!, GreenMatrix.jl:21-35
        return self.phase(lt, 1.0)[:, None] * (self.m.eK @ M)

    def wrap_forward(self, G, lt):
        d = self.phase(lt, 1.0)
        G = self.m.eK @ G @ self.m.eKinv
        return d[:, None] * G * (1.0 / d)[None, :]

    def wrap_backward(self, G, lt):
        d = self.phase(lt, -1.0)
        G = d[:, None] * G * (1.0 / d)[None, :]
        return self.m.eKinv @ G @ self.m.eK

    def update_layer(self, lt):  # UpdatePhyLayer!, phy_update.jl:188-203
        m, G, s = self.m, self.G, self.s
        for b in range(len(self.X)):
            x, y = int(self.X[b]), int(self.Y[b])
            S = [x, y]
            k, u = self.tape.draw()
            sold = int(s[b, lt - 1])
            sx = _sx(sold, k)
            Δs = m.η[sx - 1] - m.η[sold - 1]                                 # get_r!, GreenMatrix.jl:73-89
            t2 = np.array([Δs, m.a * Δs])
            t2 = np.exp(1j * t2) - 1 if m.is_complex else np.exp(t2) - 1
            r = -(t2[:, None] * G[np.ix_(S, S)])
            r[0, 0] = (t2[0] + r[0, 0]) + 1
            r[1, 1] = (t2[1] + r[1, 1]) + 1
            dt = det22(r)
            p = float(abs(dt) ** 2) if m.is_complex else float(dt * dt)
            r = inv22(r) * t2[None, :]
            p *= m.γ[sx - 1] / m.γ[sold - 1]
            if not m.is_complex:
                p *= math.exp((m.η[sold - 1] - m.η[sx - 1]) * (m.a + 1))
            acc = u < p
            self.accepts.append(acc)
            if acc:
                Gupdate(G, S, r)
                s[b, lt - 1] = sx

    def measure(self, lt):  # phy_measure, phy_update.jl:205-355 (xy_i called correctly)
        m = self.m
        G0 = self.G.copy()
        half = m.Nt // 2
        if lt > m.Nt / 2:
            for t in range(lt, half, -1):
                G0 = self.wrap_backward(G0, t)
        else:
            for t in range(lt + 1, half + 1):
                G0 = self.wrap_forward(G0, t)
        G0 = m.HalfeK @ G0 @ m.HalfeKinv
        Ek = 2 * m.Ht * np.real(np.sum(m.K * G0))
        d = np.diag(G0)
        X, Y = self.X, self.Y
        gxx, gyy, gxy, gyx = G0[X, X], G0[Y, Y], G0[X, Y], G0[Y, X]
        if m.is_complex:
            Eu = np.sum((1 - d) * d.conj())
            Ev = np.sum((1 - gxx) * (1 - gyy) - gxy * gyx + np.conj(gxx * gyy - gxy * gyx)
                        + (1 - gyy) * gxx.conj() + (1 - gxx) * gyy.conj())
        else:
            Eu = np.sum((1 - d) * (1 - d))
            Ev = np.sum(2 * ((1 - gxx) * (1 - gyy) - gxy * gyx) + 2 * (1 - gyy) * (1 - gxx))
        out = [Ek, m.U * np.real(Eu), m.V * np.real(Ev), 0.0, 0.0, 0.0, 0.0]
        if "HoneyComb" in m.Lattice:
            out[3:] = _honeycomb_sf_quirk(m.site, G0, m.Ns, spinful_real=not m.is_complex)
        if self.full_sf:
            out += _honeycomb_sf_full(m.site, G0, m.Ns) if "HoneyComb" in m.Lattice else _square_sf_full(m, G0)
        return np.array(out)

    def run(self, sweeps):
        m = self.m
        self.init_chain()
        for _ in range(sweeps):
            acc, cnt = np.zeros(11 if self.full_sf else 7), 0
            for lt in range(1, m.Nt + 1):
                self.G = self.wrap_forward(self.G, lt)
                self.update_layer(lt)
                if self.record and abs(self.idx - self.Θidx) <= 1:
                    acc += self.measure(lt)
                    cnt += 1
                if lt in self.node_set:
                    self.node_forward()
            for lt in range(m.Nt, 0, -1):
                self.update_layer(lt)
                if self.record and abs(self.idx - self.Θidx) <= 1:
                    acc += self.measure(lt)
                    cnt += 1
                self.G = self.wrap_backward(self.G, lt)
                if lt - 1 in self.node_set:
                    self.node_backward()
            if self.record:
                self.obs_rows.append(acc / cnt)
        return self


# --------------------------------------------------------------------------
# structure factors
# --------------------------------------------------------------------------
def _cells(site):
    """0-based A-site index of every unit cell (ix, iy), 1-based cell coords."""
    L1, L2 = site
    return {(ix, iy): 2 * (ix + (iy - 1) * L1) - 2 for ix in range(1, L1 + 1)
            for iy in range(1, L2 + 1)}


def _honeycomb_sf_quirk(site, G0, Ns, spinful_real):
    """CDW0, CDW1, SDW0, SDW1 on the honeycomb lattice.

    Complex branch: src/tU/phy_update.jl:194-235 and src/tUV/phy_update.jl:
    306-323, where each ``+adjoint(...)`` continuation line is a separate,
    discarded Julia statement, so only the first term of every correlator is
    accumulated.  Real branch: src/tUV/phy_update.jl:296-305 (all terms).
    """
    L1, L2 = site
    cells = _cells(site)
    CDW0 = CDW1 = SDW0 = SDW1 = 0.0
    for rx in range(1, L1 + 1):
        for ry in range(1, L2 + 1):
            t1 = t2 = 0.0
            for (ix, iy), a1 in cells.items():
                a2 = cells[((ix + rx - 1) % L1 + 1, (iy + ry - 1) % L2 + 1)]
                b1, b2 = a1 + 1, a2 + 1
                δ = 1.0 if a1 == a2 else 0.0
                g = G0
                if spinful_real:
                    t1 += 2 * ((1 - g[a1, a1]) * (1 - g[a2, a2]) + (δ - g[a1, a2]) * g[a2, a1])
                    t1 += 2 * ((1 - g[b1, b1]) * (1 - g[b2, b2]) + (δ - g[b1, b2]) * g[b2, b1])
                    t1 -= 2 * ((1 - g[b1, b1]) * (1 - g[a2, a2]) - g[b1, a2] * g[a2, b1])
                    t1 -= 2 * ((1 - g[a1, a1]) * (1 - g[b2, b2]) - g[a1, b2] * g[b2, a1])
                    t2 += 2 * (1 - g[a1, a1]) * (1 - g[a2, a2])
                    t2 += 2 * (1 - g[b1, b1]) * (1 - g[b2, b2])
                    t2 -= 2 * (1 - g[b1, b1]) * (1 - g[a2, a2])
                    t2 -= 2 * (1 - g[a1, a1]) * (1 - g[b2, b2])
                else:
                    t1 += (1 - g[a1, a1]) * (1 - g[a2, a2]) + (δ - g[a1, a2]) * g[a2, a1]
                    t1 += (1 - g[b1, b1]) * (1 - g[b2, b2]) + (δ - g[b1, b2]) * g[b2, b1]
                    t1 -= (1 - g[b1, b1]) * (1 - g[a2, a2]) - g[b1, a2] * g[a2, b1]
                    t1 -= (1 - g[a1, a1]) * (1 - g[b2, b2]) - g[a1, b2] * g[b2, a1]
                    t2 += (1 - g[a1, a1]) * np.conj(g[a2, a2])
                    t2 += (1 - g[b1, b1]) * np.conj(g[b2, b2])
                    t2 -= (1 - g[a1, a1]) * np.conj(g[b2, b2])
                    t2 -= (1 - g[b1, b1]) * np.conj(g[a2, a2])
            ph = math.cos(2 * math.pi / L1 * rx + 2 * math.pi / L2 * ry)
            CDW0 += t1 + t2
            CDW1 += ph * (t1 + t2)
            SDW0 += t1 - t2
            SDW1 += ph * (t1 - t2)
    n2 = Ns ** 2
    return [float(np.real(v)) / n2 for v in (CDW0, CDW1, SDW0, SDW1)]


def _honeycomb_sf_full(site, G0, Ns):
    """CDW0, CDW1, SDW0, SDW1 of the complex branch with every term: each
    correlator of src/tU/phy_update.jl:194-235 plus its ``+adjoint(...)``
    continuation (the opposite-spin part), which the reference discards."""
    L1, L2 = site
    cells = _cells(site)
    CDW0 = CDW1 = SDW0 = SDW1 = 0.0
    g, c = G0, np.conj
    for rx in range(1, L1 + 1):
        for ry in range(1, L2 + 1):
            t1 = t2 = 0.0
            for (ix, iy), a1 in cells.items():
                a2 = cells[((ix + rx - 1) % L1 + 1, (iy + ry - 1) % L2 + 1)]
                b1, b2 = a1 + 1, a2 + 1
                δ = 1.0 if a1 == a2 else 0.0
                t1 += (1 - g[a1, a1]) * (1 - g[a2, a2]) + (δ - g[a1, a2]) * g[a2, a1] \
                    + c(g[a1, a1] * g[a2, a2] + g[a1, a2] * (δ - g[a2, a1]))
                t1 += (1 - g[b1, b1]) * (1 - g[b2, b2]) + (δ - g[b1, b2]) * g[b2, b1] \
                    + c(g[b1, b1] * g[b2, b2] + g[b1, b2] * (δ - g[b2, b1]))
                t1 -= (1 - g[b1, b1]) * (1 - g[a2, a2]) - g[b1, a2] * g[a2, b1] \
                    + c(g[b1, b1] * g[a2, a2] - g[b1, a2] * g[a2, b1])
                t1 -= (1 - g[a1, a1]) * (1 - g[b2, b2]) - g[a1, b2] * g[b2, a1] \
                    + c(g[a1, a1] * g[b2, b2] - g[a1, b2] * g[b2, a1])
                t2 += (1 - g[a1, a1]) * c(g[a2, a2]) + c(g[a1, a1]) * (1 - g[a2, a2])
                t2 += (1 - g[b1, b1]) * c(g[b2, b2]) + c(g[b1, b1]) * (1 - g[b2, b2])
                t2 -= (1 - g[a1, a1]) * c(g[b2, b2]) + c(g[a1, a1]) * (1 - g[b2, b2])
                t2 -= (1 - g[b1, b1]) * c(g[a2, a2]) + c(g[b1, b1]) * (1 - g[a2, a2])
            ph = math.cos(2 * math.pi / L1 * rx + 2 * math.pi / L2 * ry)
            CDW0 += t1 + t2
            CDW1 += ph * (t1 + t2)
            SDW0 += t1 - t2
            SDW1 += ph * (t1 - t2)
    n2 = Ns ** 2
    return [float(np.real(v)) / n2 for v in (CDW0, CDW1, SDW0, SDW1)]


def staggered_signs(K):
    """+1 / -1 per site of a two-colouring of the hopping graph (nonzero K
    entries), site 0 on +1; all zeros when the graph is not bipartite."""
    K = np.asarray(K)
    N = K.shape[0]
    adj = np.abs(K) > 1e-12
    sign = np.zeros(N, dtype=np.int64)
    for root in range(N):
        if sign[root]:
            continue
        sign[root] = 1
        stack = [root]
        while stack:
            i = stack.pop()
            for j in np.nonzero(adj[i])[0]:
                if j == i:
                    continue
                if sign[j] == 0:
                    sign[j] = -sign[i]
                    stack.append(j)
                elif sign[j] == sign[i]:
                    return np.zeros(N, dtype=np.int64)
    return sign


def _square_sf_full(model, G0):
    """The square lattices' counterpart of the corrected honeycomb structure
    factors (no counterpart in the reference, whose square branch measures
    none): the staggered charge and spin structure factors at (pi, pi),
    sum_ij e_i e_j <(rho_i)(rho_j)> / Ns^2 with rho = n_up + n_dn (charge)
    or n_up - n_dn (spin) and e the two-colouring of the lattice, every term
    of the correlators as in the honeycomb form; the two shifted-momentum
    columns stay 0."""
    eps = staggered_signs(model.K).astype(np.float64)
    g, c = G0, np.conj
    d = np.diag(g)
    same = (1 - d)[:, None] * (1 - d)[None, :] - g * g.T + c(d[:, None] * d[None, :] - g * g.T)
    same = same + np.diag(d + c(d))            # the delta_ij terms: G_ii + conj(G_ii)
    opp = (1 - d)[:, None] * c(d)[None, :] + c(d)[:, None] * (1 - d)[None, :]
    w = eps[:, None] * eps[None, :]
    n2 = model.Ns ** 2
    return [float(np.real(np.sum(w * (same + opp)))) / n2, 0.0,
            float(np.real(np.sum(w * (same - opp)))) / n2, 0.0]


def _tv_density_sf(site, G0, Ns):
    """R0, R1 (4 sublattice components each).  src/tV/phy_update.jl:268-294."""
    L1, L2 = site
    cells = _cells(site)
    R0, R1 = np.zeros(4), np.zeros(4)
    g = G0
    for rx in range(1, L1 + 1):
        for ry in range(1, L2 + 1):
            t = np.zeros(4)
            for (ix, iy), a1 in cells.items():
                a2 = cells[((ix + rx - 1) % L1 + 1, (iy + ry - 1) % L2 + 1)]
                b1, b2 = a1 + 1, a2 + 1
                if a1 == a2:
                    t[0] += 1 - g[a1, a1]
                    t[1] += 1 - g[b1, b1]
                else:
                    t[0] += (1 - g[a1, a1]) * (1 - g[a2, a2]) - g[a1, a2] * g[a2, a1]
                    t[1] += (1 - g[b1, b1]) * (1 - g[b2, b2]) - g[b1, b2] * g[b2, b1]
                t[2] += (1 - g[b1, b1]) * (1 - g[a2, a2]) - g[b1, a2] * g[a2, b1]
                t[3] += (1 - g[a1, a1]) * (1 - g[b2, b2]) - g[a1, b2] * g[b2, a1]
            R0 += t
            R1 += math.cos(2 * math.pi / L1 * rx + 2 * math.pi / L2 * ry) * t
    return R0 * 4 / Ns ** 2, R1 * 4 / Ns ** 2


# --------------------------------------------------------------------------
# public entry points
# --------------------------------------------------------------------------
_SWEEPS = {KIND_TU: _TUSweep, KIND_TV: _TVSweep, KIND_TUV: _TUVSweep}


def proposals_per_sweep(model) -> int:
    return 2 * model.Nt * model.n_field


def phy_update(model, s, sweeps: int, tape: Tape, record: bool = False, slmc=None, full_sf: bool = False):
    """Run ``sweeps`` sweeps; returns the sweep object (s, G, accepts, drift, obs_rows).

    Mirrors ``phy_update(path, model, s, Sweeps, record)`` without the CSV side
    output: src/tU/phy_update.jl:3-152, src/tV/phy_update.jl:1-188,
    src/tUV/phy_update.jl:1-186.  ``slmc`` (t-U only) adds the cluster moves:
    a dict with params, moves, cluster_len, steps, seed and chain.
    """
    sw = _SWEEPS[model.kind](model, s, tape, record)
    sw.full_sf = full_sf
    if slmc is not None:
        if model.kind != KIND_TU:
            raise ValueError("cluster moves are restated for t-U only")
        sw.slmc = slmc
    return sw.run(sweeps)


def G_tau(model, s, τ: int):
    """Brute-force equal-time G at slice τ with QR every BatchSize slices.

    Debug oracle of the reference: src/tU/GreenMatrix.jl:91-123,
    src/tV/GreenMatrix.jl:124-194, src/tUV/GreenMatrix.jl:128-179.
    """
    sw = _SWEEPS[model.kind](model, s, Tape([], []), False)
    dt = sw.dtype
    BL = model.Pt.conj().T.astype(dt)
    BR = model.Pt.astype(dt)
    cnt = 0
    for i in range(model.Nt, τ, -1):
        BL = BL @ sw.B_left(i, np.eye(model.Ns, dtype=dt))
        cnt += 1
        if cnt == model.BatchSize:
            cnt = 0
            BL = np.linalg.qr(BL.conj().T)[0].conj().T
    cnt = 0
    for i in range(1, τ + 1):
        BR = sw.B_left(i, BR)
        cnt += 1
        if cnt == model.BatchSize:
            cnt = 0
            BR = np.linalg.qr(BR)[0]
    BL = np.linalg.qr(BL.conj().T)[0].conj().T
    BR = np.linalg.qr(BR)[0]
    return np.eye(model.Ns) - BR @ np.linalg.inv(BL @ BR) @ BL


def log_det(model, s):
    """log|det(P^H B(Theta,0) P)| and det/|det| of the fields ``s``.

    B(Theta,0) is the product of all Nt slice matrices (BM_F!, src/tU/
    GreenMatrix.jl:10-27 and siblings), applied to P from the left with a QR
    every BatchSize slices as in the reference's right chain
    (src/tU/phy_update.jl:84-87); the log|R_jj| and phases of the dropped
    triangles, which the reference discards, are summed here.
    """
    sw = _SWEEPS[model.kind](model, s, Tape([], []), False)
    dt = sw.dtype
    BR = model.Pt.astype(dt)
    lg, ph = 0.0, 1.0 + 0j
    cnt = 0
    for i in range(1, model.Nt + 1):
        BR = sw.B_left(i, BR)
        cnt += 1
        if cnt == model.BatchSize or i == model.Nt:
            cnt = 0
            Q, R = np.linalg.qr(BR)
            d = np.diag(R)
            lg += float(np.log(np.abs(d)).sum())
            ph *= complex(np.prod(d / np.abs(d)))
            BR = Q
    sgn, lm = np.linalg.slogdet(model.Pt.conj().T.astype(dt) @ BR)
    return lg + float(lm), complex(ph * sgn)


def log_weight(model, s):
    """log|W(s)|: the local HS weights times the determinant part whose ratios
    the sweep accepts with (src/tU/phy_update.jl:260-261; src/tV/GreenMatrix.jl:
    76-89 and src/tV/phy_update.jl:196-199; src/tUV/GreenMatrix.jl:73-89 and
    src/tUV/phy_update.jl:192-197): |det|^2 for t-U and complex t-UV, det for
    t-V, det^2 with e^{-(a+1) eta} for real t-UV."""
    ld, _ = log_det(model, s)
    idx = np.asarray(s).astype(np.int64).ravel() - 1
    loc = 0.0
    for i in idx:
        loc += math.log(model.γ[i])
        if model.kind == KIND_TUV and not model.is_complex:
            loc -= (model.a + 1.0) * model.η[i]
    return loc + (ld if model.kind == KIND_TV else 2.0 * ld)


def grover_det(G1, G2, index):
    """det of the Grover matrix on region A: 2 G1 G2 - G1 - G2 + I.

    src/public/GF.jl:101-109 and ``det`` in get_ABGM! (src/tU/SCEE.jl:264-276).
    ``index`` holds 1-based site indices.
    """
    ix = np.asarray(index) - 1
    A, B = G1[np.ix_(ix, ix)], G2[np.ix_(ix, ix)]
    g = 2 * A @ B - A - B + np.eye(len(ix))
    return np.linalg.det(g)
