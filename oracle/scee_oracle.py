"""CPU restatement of KAPDQMC's coupled incremental SCEE sweep (t-U).

TEST INFRASTRUCTURE ONLY: the checker of the CUDA SCEE sweep; the product
never calls it.

``ctrl_SCEEicr`` (src/tU/SCEE.jl:1-262) runs two replicas of the t-U field
whose weight is reweighted by the Rényi-2 Grover determinants of two regions,
|det g_A|^(2 λ) |det g_B|^(2 (1 - λ)), and records the mean over slices of
(|det g_A|^2 / |det g_B|^2)^(1/Nλ) per sweep (the incremental estimator of
exp(-ΔS2)).  Each replica keeps four Green's functions (G4Buffer_,
src/public/Buffer.jl:22-31): Gt = G(τ, τ), G0 = G(τ0, τ0) at the middle node,
Gt0 = G(τ, τ0), G0t = G(τ0, τ), and the inverse Grover matrices of A and B
are kept up to date by rank-1 updates.  Numerics follow src/public/Gupdate.jl
(G4! :159-212, G4update! :23-37, get_abTau1!/2! :91-132, GMupdate! :45-58)
and src/tU/SCEE.jl (get_ABGM! :264-276, UpdateSCEELayer! :278-324), with the
random draws taken from an explicit tape in the reference's consumption
order: per site, replica 1's (choice, uniform) then replica 2's.
"""
from __future__ import annotations

import numpy as np

import dqmc_oracle as O


class SCEE:
    def __init__(self, model, s1, s2, indexA, indexB, lam: float, nlam: int, tape: O.Tape):
        self.m = model
        self.s = [np.array(s1, dtype=np.uint8, order="F", copy=True),
                  np.array(s2, dtype=np.uint8, order="F", copy=True)]
        self.A = np.asarray(indexA, dtype=np.int64) - 1
        self.B = np.asarray(indexB, dtype=np.int64) - 1
        self.lam, self.nlam, self.tape = lam, nlam, tape
        self.nodes = [int(v) for v in model.nodes]
        self.NN = len(self.nodes)
        self.Θ = self.NN // 2 + 1
        self.I = np.eye(model.Ns, dtype=np.complex128)
        self.accepts: list = []
        self.O: list = []
        self.nrep = 2

    # slice matrices (BM_F!, BMinv_F!: src/tU/GreenMatrix.jl:10-47) --------
    def D(self, r, lt, sign=1.0):
        m = self.m
        return np.exp(1j * sign * m.α[lt - 1] * m.η[self.s[r][:, lt - 1].astype(np.int64) - 1])

    def BM(self, r, idx):
        M = self.I.copy()
        for lt in range(self.nodes[idx - 1] + 1, self.nodes[idx] + 1):
            M = self.D(r, lt)[:, None] * (self.m.eK @ M)
        return M

    def BMinv(self, r, idx):
        M = self.I.copy()
        for lt in range(self.nodes[idx - 1] + 1, self.nodes[idx] + 1):
            M = (M @ self.m.eKinv) * self.D(r, lt, -1.0)[None, :]
        return M

    # four Green's functions at node idx (G4!) ------------------------------
    def G4(self, r, idx, forward: bool):
        BL, BR, BMs, BMi = self.BL[r], self.BR[r], self.BMs[r], self.BMi[r]
        Θ, I = self.Θ, self.I
        Gt = O.get_G(BL[idx], BR[idx])
        if idx == Θ:
            G0 = Gt.copy()
            Gt0, G0t = (Gt.copy(), Gt - I) if forward else (Gt - I, Gt.copy())
        else:
            G0 = O.get_G(BL[Θ], BR[Θ])
            Gt0, G0t = I.copy(), I.copy()
            if idx < Θ:
                for j in range(idx, Θ):
                    Gj = Gt if j == idx else O.get_G(BL[j], BR[j])
                    G0t = BMs[j] @ (Gj @ G0t)
                    Gt0 = (Gt0 @ (I - Gj)) @ BMi[j]
                Gt0 = -Gt0
            else:
                for j in range(Θ, idx):
                    Gj = G0 if j == Θ else O.get_G(BL[j], BR[j])
                    Gt0 = BMs[j] @ (Gj @ Gt0)
                    G0t = (G0t @ (I - Gj)) @ BMi[j]
                G0t = -G0t
        self.Gt[r], self.G0[r], self.Gt0[r], self.G0t[r] = Gt, G0, Gt0, G0t

    def grover(self, idx_region):
        a = self.G0[0][np.ix_(idx_region, idx_region)]
        b = self.G0[1][np.ix_(idx_region, idx_region)]
        g = 2 * a @ b - a - b + np.eye(len(idx_region))
        return abs(np.linalg.det(g)) ** 2, np.linalg.inv(g)

    def ABGM(self, idx, forward):   # get_ABGM!, src/tU/SCEE.jl:264-276
        self.G4(0, idx, forward)
        self.G4(1, idx, forward)
        self.detA, self.invA = self.grover(self.A)
        self.detB, self.invB = self.grover(self.B)

    # one replica's proposal at site i ----------------------------------------
    def propose(self, r, lt, i):
        m, s = self.m, self.s[r]
        k, u = self.tape.draw()
        sold = int(s[i, lt - 1])
        sx = O._sx(sold, k)
        Δ = np.exp(1j * m.α[lt - 1] * (m.η[sx - 1] - m.η[sold - 1])) - 1     # get_r!
        Gt, Gt0, G0t = self.Gt[r], self.Gt0[r], self.G0t[r]
        pc = 1 + Δ * (1 - Gt[i, i])
        rr = Δ / pc
        p = abs(pc) ** 2 * m.γ[sx - 1] / m.γ[sold - 1]
        other = self.G0[1 - r]
        taus = []
        for reg, inv in ((self.A, self.invA), (self.B, self.invB)):
            X = 2 * other[np.ix_(reg, reg)] - np.eye(len(reg))
            if r == 0:   # get_abTau1!
                a = G0t[reg, i] * rr
                b = (Gt0[i, reg] @ X) @ inv
            else:        # get_abTau2!
                a = X @ G0t[reg, i]
                b = (rr * Gt0[i, reg]) @ inv
            taus.append((a, b, 1 + b @ a))
        dA, dB = abs(taus[0][2]) ** 2, abs(taus[1][2]) ** 2
        p *= dA ** self.lam * dB ** (1 - self.lam)
        acc = u < p
        self.accepts.append(bool(acc))
        if acc:
            self.detA *= dA
            self.detB *= dB
            for (a, b, tau), name in zip(taus, ("invA", "invB")):   # GMupdate!
                inv = getattr(self, name)
                setattr(self, name, inv - np.outer(inv @ a, b) / tau)
            G0 = self.G0[r]                                           # G4update!
            zN = rr * Gt0[i, :]
            c0t, ct = G0t[:, i].copy(), Gt[:, i].copy()
            G0 += np.outer(c0t, zN)
            Gt0 += np.outer(ct, zN)
            zN = -rr * Gt[i, :]
            zN[i] += rr
            G0t -= np.outer(c0t, zN)
            Gt -= np.outer(ct, zN)
            s[i, lt - 1] = sx

    def layer(self, lt):   # UpdateSCEELayer!, src/tU/SCEE.jl:278-324
        for i in range(self.m.Ns):
            self.propose(0, lt, i)
            self.propose(1, lt, i)

    def wrap(self, r, lt, forward: bool):   # WrapKV! "L", "B", "R" (src/tU/GreenMatrix.jl:56-86)
        m = self.m
        if forward:
            d = self.D(r, lt)
            self.Gt0[r] = d[:, None] * (m.eK @ self.Gt0[r])
            self.Gt[r] = d[:, None] * (m.eK @ self.Gt[r] @ m.eKinv) / d[None, :]
            self.G0t[r] = (self.G0t[r] @ m.eKinv) / d[None, :]
        else:
            d = self.D(r, lt)
            self.Gt0[r] = m.eKinv @ (self.Gt0[r] / d[:, None])
            self.Gt[r] = m.eKinv @ ((self.Gt[r] / d[:, None]) * d[None, :]) @ m.eK
            self.G0t[r] = (self.G0t[r] * d[None, :]) @ m.eK

    def init(self):
        NN = self.NN
        self.BMs = [[None] * (NN + 1) for _ in range(2)]
        self.BMi = [[None] * (NN + 1) for _ in range(2)]
        self.BL = [[None] * (NN + 1) for _ in range(2)]
        self.BR = [[None] * (NN + 1) for _ in range(2)]
        self.Gt, self.G0, self.Gt0, self.G0t = [None] * 2, [None] * 2, [None] * 2, [None] * 2
        Pt = self.m.Pt.astype(self.I.dtype)
        for r in range(self.nrep):
            for idx in range(1, NN):
                self.BMs[r][idx] = self.BM(r, idx)
                self.BMi[r][idx] = self.BMinv(r, idx)
            self.BL[r][NN] = Pt.conj().T
            self.BR[r][1] = Pt.copy()
            for i in range(1, NN):
                self.BL[r][NN - i] = O.orth_rows(self.BL[r][NN - i + 1] @ self.BMs[r][NN - i])
                self.BR[r][i + 1] = O.orth_cols(self.BMs[r][i] @ self.BR[r][i])
        self.idx = 1
        self.ABGM(1, True)
        return self

    def forward_slice(self, lt):
        Θ = self.Θ
        for r in range(self.nrep):
            self.wrap(r, lt, True)
        self.layer(lt)
        val = (self.detA / self.detB) ** (1 / self.nlam)
        if lt in self.nodes:
            self.idx += 1
            idx = self.idx
            for r in range(self.nrep):
                self.BMs[r][idx - 1] = self.BM(r, idx - 1)
                self.BMi[r][idx - 1] = self.BMinv(r, idx - 1)
                for i in range(idx, max(Θ, idx) + 1):
                    self.BR[r][i] = O.orth_cols(self.BMs[r][i - 1] @ self.BR[r][i - 1])
                for i in range(idx - 1, min(Θ, idx) - 1, -1):
                    self.BL[r][i] = O.orth_rows(self.BL[r][i + 1] @ self.BMs[r][i])
            self.ABGM(idx, True)
        return val

    def backward_slice(self, lt):
        Θ = self.Θ
        self.layer(lt)
        val = (self.detA / self.detB) ** (1 / self.nlam)
        if (lt - 1) in self.nodes:
            self.idx -= 1
            idx = self.idx
            for r in range(self.nrep):
                self.BMs[r][idx] = self.BM(r, idx)
                self.BMi[r][idx] = self.BMinv(r, idx)
                for i in range(idx, min(Θ, idx) - 1, -1):
                    self.BL[r][i] = O.orth_rows(self.BL[r][i + 1] @ self.BMs[r][i])
                for i in range(idx + 1, max(Θ, idx) + 1):
                    self.BR[r][i] = O.orth_cols(self.BMs[r][i - 1] @ self.BR[r][i - 1])
            self.ABGM(idx, False)
        else:
            for r in range(self.nrep):
                self.wrap(r, lt, False)
        return val

    def run(self, sweeps: int):
        """src/tU/SCEE.jl:89-246: forward then backward over the slices, the
        estimator accumulated after every slice's updates."""
        self.init()
        for _ in range(sweeps):
            vals = [self.forward_slice(lt) for lt in range(1, self.m.Nt + 1)]
            vals += [self.backward_slice(lt) for lt in range(self.m.Nt, 0, -1)]
            self.O.append(float(np.mean(vals)))
        return self


def proposals_per_sweep(model) -> int:
    return 4 * model.Ns * model.Nt


def ctrl_SCDOPicr(model, alpha, indexA, indexB, sweeps, lam, nlam, s, tape: O.Tape):
    """Disorder-operator sweep of the field ``s``; returns the DOP object."""
    return DOP(model, s, alpha, indexA, indexB, lam, nlam, tape).run(sweeps)


def ctrl_SCEEicr(model, indexA, indexB, sweeps, lam, nlam, ss, tape: O.Tape):
    """Run ``sweeps`` coupled sweeps of the replica pair ``ss``; returns the
    SCEE object (fields ``s``, ``O`` per sweep, Green's functions, accepts)."""
    return SCEE(model, ss[0], ss[1], indexA, indexB, lam, nlam, tape).run(sweeps)


class DOP(SCEE):
    """ctrl_SCDOPicr (src/tU/disorder_operate.jl:1-247): one replica, its
    weight reweighted by |det X_A|^(2 λ) |det X_B|^(2 (1 - λ)) with the
    disorder-operator matrices X = e^{iα} I + (1 - e^{iα}) G0[R,R] (get_ABX!,
    :202-224); the estimator is (|det X_A|^2 / |det X_B|^2)^(1/Nλ).  Updates
    follow UpdateSCDOPLayer! (:225-247) with get_abTau! for DOPBuffer_
    (src/public/Gupdate.jl:60-81): a = (1 - e^{iα}) G0t[R,i] r,
    b = Gt0[i,R] Xinv, Tau = 1 + b a."""

    def __init__(self, model, s, alpha, indexA, indexB, lam, nlam, tape):
        super().__init__(model, s, s, indexA, indexB, lam, nlam, tape)
        self.s = self.s[:1]
        self.alpha = alpha
        self.nrep = 1

    def xmat(self, reg):
        e = np.exp(1j * self.alpha)
        X = (1 - e) * self.G0[0][np.ix_(reg, reg)] + e * np.eye(len(reg))
        return abs(np.linalg.det(X)) ** 2, np.linalg.inv(X)

    def ABGM(self, idx, forward):   # get_ABX!
        self.G4(0, idx, forward)
        self.detA, self.invA = self.xmat(self.A)
        self.detB, self.invB = self.xmat(self.B)

    def propose(self, r, lt, i):
        m, s = self.m, self.s[0]
        k, u = self.tape.draw()
        sold = int(s[i, lt - 1])
        sx = O._sx(sold, k)
        Δ = np.exp(1j * m.α[lt - 1] * (m.η[sx - 1] - m.η[sold - 1])) - 1
        Gt, Gt0, G0t = self.Gt[0], self.Gt0[0], self.G0t[0]
        pc = 1 + Δ * (1 - Gt[i, i])
        rr = Δ / pc
        p = abs(pc) ** 2 * m.γ[sx - 1] / m.γ[sold - 1]
        e = np.exp(1j * self.alpha)
        taus = []
        for reg, inv in ((self.A, self.invA), (self.B, self.invB)):
            a = (1 - e) * (G0t[reg, i] * rr)
            b = Gt0[i, reg] @ inv
            taus.append((a, b, 1 + b @ a))
        dA, dB = abs(taus[0][2]) ** 2, abs(taus[1][2]) ** 2
        p *= dA ** self.lam * dB ** (1 - self.lam)
        acc = u < p
        self.accepts.append(bool(acc))
        if acc:
            self.detA *= dA
            self.detB *= dB
            for (a, b, tau), name in zip(taus, ("invA", "invB")):
                inv = getattr(self, name)
                setattr(self, name, inv - np.outer(inv @ a, b) / tau)
            G0 = self.G0[0]
            zN = rr * Gt0[i, :]
            c0t, ct = G0t[:, i].copy(), Gt[:, i].copy()
            G0 += np.outer(c0t, zN)
            Gt0 += np.outer(ct, zN)
            zN = -rr * Gt[i, :]
            zN[i] += rr
            G0t -= np.outer(c0t, zN)
            Gt -= np.outer(ct, zN)
            s[i, lt - 1] = sx

    def layer(self, lt):   # UpdateSCDOPLayer!
        for i in range(self.m.Ns):
            self.propose(0, lt, i)


class SCEE_TV(SCEE):
    """ctrl_SCEEicr for t-V (src/tV/SCEE.jl:1-517): real arithmetic, bond
    fields, rank-2 updates with 2x2 Tau matrices, the Grover determinant
    itself (not its modulus squared) in the weight, and the bond rotations
    wrapped direction by direction between the updates of each direction
    (WrapK! :509-517, WrapV! src/tV/GreenMatrix.jl:99-119)."""

    def __init__(self, model, s1, s2, indexA, indexB, lam, nlam, tape):
        super().__init__(model, s1, s2, indexA, indexB, lam, nlam, tape)
        self.I = np.eye(model.Ns)
        self.tv = []
        for r in range(2):
            sw = O._TVSweep(model, self.s[r], O.Tape([], []), False)
            sw.s = self.s[r]          # share the replica's live field
            self.tv.append(sw)

    def BM(self, r, idx):   # BM_F!, src/tV/GreenMatrix.jl:12-38
        M = self.I.copy()
        for lt in range(self.nodes[idx - 1] + 1, self.nodes[idx] + 1):
            M = self.tv[r].B_left(lt, M)
        return M

    def BMinv(self, r, idx):   # BMinv_F!, src/tV/GreenMatrix.jl:40-66
        sw, M = self.tv[r], self.I.copy()
        for lt in range(self.nodes[idx - 1] + 1, self.nodes[idx] + 1):
            M = M @ self.m.eKinv
            for j in reversed(range(self.m.z)):
                M = sw.uvR(j, sw.uvR(j, M) * sw.Dj(lt, j, -1.0)[None, :])
        return M

    def grover(self, reg):   # get_ABGM!, src/tV/SCEE.jl:433-445: det, not its modulus squared
        a = self.G0[0][np.ix_(reg, reg)]
        b = self.G0[1][np.ix_(reg, reg)]
        g = 2 * a @ b - a - b + np.eye(len(reg))
        return float(np.linalg.det(g)), np.linalg.inv(g)

    def wrapK(self, r, forward):   # WrapK!
        m = self.m
        A, Ai = (m.eK, m.eKinv) if forward else (m.eKinv, m.eK)
        self.Gt[r] = A @ self.Gt[r] @ Ai
        self.Gt0[r] = A @ self.Gt0[r]
        self.G0t[r] = self.G0t[r] @ Ai

    def wrapV(self, r, lt, j, forward):   # WrapV! "L", "B", "R" of direction j
        sw = self.tv[r]
        d = sw.Dj(lt, j, 1.0 if forward else -1.0)
        self.Gt0[r] = sw.uvL(j, d[:, None] * sw.uvL(j, self.Gt0[r]))
        self.Gt[r] = sw.wrapV(self.Gt[r], j, d)
        self.G0t[r] = sw.uvR(j, sw.uvR(j, self.G0t[r]) / d[None, :])

    def propose_bond(self, r, lt, j, i):   # UpdateSCEELayer!, src/tV/SCEE.jl:447-508
        m, s, sw = self.m, self.s[r], self.tv[r]
        x, y = int(sw.X[j][i]), int(sw.Y[j][i])
        S = [x, y]
        k, u = self.tape.draw()
        sold = int(s[i, j, lt - 1])
        sx = O._sx(sold, k)
        Δs = m.α[lt - 1] * (m.η[sx - 1] - m.η[sold - 1])                    # get_r!
        t2 = np.exp(Δs * np.array([1.0, -1.0])) - 1
        Δ = (sw.uv * t2[None, :]) @ sw.uv
        Gt, Gt0, G0t = self.Gt[r], self.Gt0[r], self.G0t[r]
        rm = Δ - Δ @ Gt[np.ix_(S, S)]
        rm[0, 0] += 1
        rm[1, 1] += 1
        p = O.det22(rm)
        rr = O.inv22(rm) @ Δ
        p *= m.γ[sx - 1] / m.γ[sold - 1]
        other = self.G0[1 - r]
        taus = []
        for reg, inv in ((self.A, self.invA), (self.B, self.invB)):
            X = 2 * other[np.ix_(reg, reg)] - np.eye(len(reg))
            if r == 0:   # get_abTau1!
                a = G0t[np.ix_(reg, S)] @ rr
                b = (Gt0[np.ix_(S, reg)] @ X) @ inv
            else:        # get_abTau2!
                a = X @ G0t[np.ix_(reg, S)]
                b = (rr @ Gt0[np.ix_(S, reg)]) @ inv
            tau = b @ a + np.eye(2)
            taus.append((a, b, tau, O.det22(tau)))
        dA, dB = taus[0][3], taus[1][3]
        p *= np.power(dA, self.lam) * np.power(dB, 1 - self.lam)
        self.last_p = p
        acc = u < p
        self.accepts.append(bool(acc))
        if acc:
            self.detA *= dA
            self.detB *= dB
            for (a, b, tau, _), name in zip(taus, ("invA", "invB")):   # GMupdate!
                inv = getattr(self, name)
                setattr(self, name, inv - (inv @ a) @ O.inv22(tau) @ b)
            G0 = self.G0[r]                                             # G4update!
            zN = rr @ Gt0[S, :]
            c0t, ct = G0t[:, S].copy(), Gt[:, S].copy()
            G0 += c0t @ zN
            Gt0 += ct @ zN
            zN = -rr @ Gt[S, :]
            zN[:, S] += rr
            G0t -= c0t @ zN
            Gt -= ct @ zN
            s[i, j, lt - 1] = sx

    def layer_dir(self, lt, j):
        for i in range(self.m.Ns // 2):
            self.propose_bond(0, lt, j, i)
            self.propose_bond(1, lt, j, i)

    def estimator(self):
        return np.power(self.detA / self.detB, 1 / self.nlam)

    def forward_slice(self, lt):   # src/tV/SCEE.jl:87-152
        for r in range(2):
            self.wrapK(r, True)
        for j in reversed(range(self.m.z)):
            for r in range(2):
                self.wrapV(r, lt, j, True)
            self.layer_dir(lt, j)
        val = self.estimator()
        if lt in self.nodes:
            self.node_step(forward=True)
        return val

    def backward_slice(self, lt):   # src/tV/SCEE.jl:258-330
        for j in range(self.m.z):
            self.layer_dir(lt, j)
            for r in range(2):
                self.wrapV(r, lt, j, False)
        for r in range(2):
            self.wrapK(r, False)
        val = self.estimator()
        if (lt - 1) in self.nodes:
            self.node_step(forward=False)
        return val

    def node_step(self, forward):
        Θ = self.Θ
        if forward:
            self.idx += 1
            idx = self.idx
            for r in range(2):
                self.BMs[r][idx - 1] = self.BM(r, idx - 1)
                self.BMi[r][idx - 1] = self.BMinv(r, idx - 1)
                for i in range(idx, max(Θ, idx) + 1):
                    self.BR[r][i] = O.orth_cols(self.BMs[r][i - 1] @ self.BR[r][i - 1])
                for i in range(idx - 1, min(Θ, idx) - 1, -1):
                    self.BL[r][i] = O.orth_rows(self.BL[r][i + 1] @ self.BMs[r][i])
        else:
            self.idx -= 1
            idx = self.idx
            for r in range(2):
                self.BMs[r][idx] = self.BM(r, idx)
                self.BMi[r][idx] = self.BMinv(r, idx)
                for i in range(idx, min(Θ, idx) - 1, -1):
                    self.BL[r][i] = O.orth_rows(self.BL[r][i + 1] @ self.BMs[r][i])
                for i in range(idx + 1, max(Θ, idx) + 1):
                    self.BR[r][i] = O.orth_cols(self.BMs[r][i - 1] @ self.BR[r][i - 1])
        self.ABGM(self.idx, forward)


def proposals_per_sweep_tv(model) -> int:
    return 2 * 2 * (model.Ns // 2) * model.z * model.Nt


class SCEE_TUV(SCEE):
    """ctrl_SCEEicr for t-UV (src/tUV/SCEE.jl:1-402): site phases summed over
    the bonds (eta on the bond's first site, a eta on its second), the same
    one- and two-sided slice wraps as t-U, rank-2 bond proposals with
    |det Tau|^2 factors and |det g|^2 Grover weights.  As in the reference's
    UpdateSCEELayer! (:355-402) the real-type extra weight
    exp((eta - eta')(a + 1)) of the plain sweep is not applied, and the
    backward sweep wraps every slice before the node step (:225-275)."""

    def __init__(self, model, s1, s2, indexA, indexB, lam, nlam, tape):
        super().__init__(model, s1, s2, indexA, indexB, lam, nlam, tape)
        dt = np.complex128 if model.is_complex else np.float64
        self.I = np.eye(model.Ns, dtype=dt)
        self.uv = []
        for r in range(2):
            sw = O._TUVSweep(model, self.s[r], O.Tape([], []), False)
            sw.s = self.s[r]
            self.uv.append(sw)

    def D(self, r, lt, sign=1.0):
        return self.uv[r].phase(lt, sign)

    def propose_bond(self, r, lt, b):
        m, s, sw = self.m, self.s[r], self.uv[r]
        x, y = int(sw.X[b]), int(sw.Y[b])
        S = [x, y]
        k, u = self.tape.draw()
        sold = int(s[b, lt - 1])
        sx = O._sx(sold, k)
        Δs = m.η[sx - 1] - m.η[sold - 1]                                     # get_r!
        t2 = np.array([Δs, m.a * Δs])
        t2 = np.exp(1j * t2) - 1 if m.is_complex else np.exp(t2) - 1
        Gt, Gt0, G0t = self.Gt[r], self.Gt0[r], self.G0t[r]
        rm = -(t2[:, None] * Gt[np.ix_(S, S)])
        rm[0, 0] = (t2[0] + rm[0, 0]) + 1
        rm[1, 1] = (t2[1] + rm[1, 1]) + 1
        p = abs(O.det22(rm)) ** 2
        rr = O.inv22(rm) * t2[None, :]
        p *= m.γ[sx - 1] / m.γ[sold - 1]
        other = self.G0[1 - r]
        taus = []
        for reg, inv in ((self.A, self.invA), (self.B, self.invB)):
            X = 2 * other[np.ix_(reg, reg)] - np.eye(len(reg))
            if r == 0:
                a = G0t[np.ix_(reg, S)] @ rr
                b_ = (Gt0[np.ix_(S, reg)] @ X) @ inv
            else:
                a = X @ G0t[np.ix_(reg, S)]
                b_ = (rr @ Gt0[np.ix_(S, reg)]) @ inv
            tau = b_ @ a + np.eye(2)
            taus.append((a, b_, tau, abs(O.det22(tau)) ** 2))
        dA, dB = taus[0][3], taus[1][3]
        p *= dA ** self.lam * dB ** (1 - self.lam)
        self.last_p = p
        acc = u < p
        self.accepts.append(bool(acc))
        if acc:
            self.detA *= dA
            self.detB *= dB
            for (a, b_, tau, _), name in zip(taus, ("invA", "invB")):
                inv = getattr(self, name)
                setattr(self, name, inv - (inv @ a) @ O.inv22(tau) @ b_)
            G0 = self.G0[r]
            zN = rr @ Gt0[S, :]
            c0t, ct = G0t[:, S].copy(), Gt[:, S].copy()
            G0 += c0t @ zN
            Gt0 += ct @ zN
            zN = -rr @ Gt[S, :]
            zN[:, S] += rr
            G0t -= c0t @ zN
            Gt -= ct @ zN
            s[b, lt - 1] = sx

    def layer(self, lt):
        for b in range(len(self.uv[0].X)):
            self.propose_bond(0, lt, b)
            self.propose_bond(1, lt, b)

    def backward_slice(self, lt):   # wraps before the node step
        self.layer(lt)
        val = (self.detA / self.detB) ** (1 / self.nlam)
        for r in range(2):
            self.wrap(r, lt, False)
        if (lt - 1) in self.nodes:
            SCEE_TV.node_step(self, forward=False)
        return val
