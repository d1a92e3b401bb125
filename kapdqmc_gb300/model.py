"""Model structs and keyword constructors for the t-U, t-V and t-UV models.

These mirror the reference's ``*_Hubbard_Para`` constructors field for field
(same names, same meaning, Julia column-major layouts) because they are the
drop-in boundary of the sweep: a caller builds a model here (or in Julia) and
hands its arrays to the CUDA library through the C ABI.  All of this runs on
the host, once per model.

References (KAPDQMC):
  src/tU/model.jl:14-96    tU_Hubbard_Para_ / tU_Hubbard_Para
  src/tV/model.jl:3-122    tV_Hubbard_Para_ / tV_Hubbard_Para
  src/tUV/model.jl:3-118   tUV_Hubbard_Para_ / tUV_Hubbard_Para
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from fractions import Fraction

import numpy as np

from .geometry import LATTICES, nnK_Matrix, nnidx_F

# 4-valued SU(2) Hubbard-Stratonovich constants, src/tU/model.jl:55-56
_S6 = math.sqrt(6.0)
GAMMA = np.array([1 + _S6 / 3, 1 + _S6 / 3, 1 - _S6 / 3, 1 - _S6 / 3])
ETA = np.array([math.sqrt(2 * (3 - _S6)), -math.sqrt(2 * (3 - _S6)),
                math.sqrt(2 * (3 + _S6)), -math.sqrt(2 * (3 + _S6))])

KIND_TU, KIND_TV, KIND_TUV = 0, 1, 2


def _nodes(Nt: int, BatchSize: int) -> np.ndarray:
    """Stabilisation nodes, symmetric about Nt/2.  src/tU/model.jl:81-85."""
    half = Nt // 2
    if half % BatchSize == 0:
        return np.arange(0, Nt + 1, BatchSize, dtype=np.int64)
    left = list(range(half - BatchSize, 0, -BatchSize))[::-1]
    right = list(range(half, Nt + 1, BatchSize))
    return np.array([0] + left + right + [Nt], dtype=np.int64)


def _linrange(a: float, b: float, n: int) -> np.ndarray:
    """Julia ``LinRange(a, b, n)`` element values ((1-t)a + t b, t=j/(n-1))."""
    d = n - 1
    return np.array([(1 - j / d) * a + (j / d) * b for j in range(n)])


def _profile(H1: float, H2: float, Θrelax: float, Θquench: float, Δt: float, Nt: int):
    """Interaction strength per slice, constant or a symmetric quench ramp.

    src/tU/model.jl:41-52 (tU) and src/tV/model.jl:79-90 (tV).
    """
    if Θquench > 0.0 and abs(H1 - H2) > 0:
        ramp = _linrange(H1, H2, round(Θquench / Δt) + 1)[1:]
        nr = round(Θrelax / Δt)
        H = np.concatenate([np.full(nr, H1), ramp, ramp[::-1], np.full(nr, H1)])
    else:
        if not (H1 == H2 and Θquench < 1e-7):
            raise AssertionError("For Θquench=0, H1 must equal H2")
        H = H1 * np.ones(Nt)
    if np.linalg.norm(H[::-1] - H) >= 1e-10:
        raise AssertionError("interaction profile is not symmetric!")
    if len(H) != Nt:
        raise AssertionError("Length of interaction profile does not match Nt!")
    return H


def _kinetic(HK: np.ndarray, Δt: float):
    """HalfeK, eK, HalfeKinv, eKinv from the eigendecomposition of HK.

    src/tU/model.jl:61-66 (``syevd`` then ``V * Diagonal(exp(..)) * V'``).
    """
    E, V = np.linalg.eigh(HK)
    Vh = V.conj().T

    def f(c):
        return (V * np.exp(c * E)[None, :]) @ Vh

    HalfeK, eK, HalfeKinv, eKinv = f(-Δt / 2), f(-Δt), f(Δt / 2), f(Δt)
    if np.linalg.norm(eK @ eKinv - np.eye(len(E))) >= 1e-10:
        raise AssertionError("eK*eKinv does not equal identity!")
    return HalfeK, eK, HalfeKinv, eKinv


def _stagger(Ns: int) -> np.ndarray:
    return np.diag(np.tile([-1.0, 1.0], Ns // 2))


@dataclass
class _ModelBase:
    Lattice: str
    site: list
    Ns: int
    Nt: int
    K: np.ndarray
    BatchSize: int
    Δt: float
    γ: np.ndarray
    η: np.ndarray
    Pt: np.ndarray
    HalfeK: np.ndarray
    eK: np.ndarray
    HalfeKinv: np.ndarray
    eKinv: np.ndarray
    nodes: np.ndarray

    # -- derived quantities used by the C ABI ------------------------------
    @property
    def ns(self) -> int:
        return self.Ns // 2

    @property
    def kind(self) -> int:  # pragma: no cover - overridden
        raise NotImplementedError

    @property
    def is_complex(self) -> bool:  # arithmetic type of G in the sweep
        raise NotImplementedError

    @property
    def field_shape(self) -> tuple:
        raise NotImplementedError

    @property
    def n_field(self) -> int:
        """HS field entries per time slice."""
        return int(np.prod(self.field_shape[:-1]))


@dataclass
class tU_Hubbard_Para_(_ModelBase):
    """t-U Hubbard model, complex sweep.  src/tU/model.jl:14-37."""
    Ht: float = 1.0
    Hu1: float = 0.0
    Hu2: float = 0.0
    Θrelax: float = 0.0
    Θquench: float = 0.0
    α: np.ndarray = field(default=None)

    kind = KIND_TU
    is_complex = True
    z = 1

    @property
    def field_shape(self):
        return (self.Ns, self.Nt)


@dataclass
class tV_Hubbard_Para_(_ModelBase):
    """Spinless t-V model, real sweep.  src/tV/model.jl:3-28."""
    Ht: float = 1.0
    Hv1: float = 0.0
    Hv2: float = 0.0
    Θrelax: float = 0.0
    Θquench: float = 0.0
    α: np.ndarray = field(default=None)
    nnidx: np.ndarray = field(default=None)   # (Ns/2, z, 2) 1-based
    UV: np.ndarray = field(default=None)      # (Ns, Ns, z)

    kind = KIND_TV
    is_complex = False

    @property
    def z(self) -> int:
        return self.nnidx.shape[1]

    @property
    def field_shape(self):
        return (self.Ns // 2, self.z, self.Nt)


@dataclass
class tUV_Hubbard_Para_(_ModelBase):
    """t-U-V model with bond HS fields.  src/tUV/model.jl:3-27."""
    Ht: float = 1.0
    U: float = 0.0
    V: float = 0.0
    a: float = 0.0
    Type: type = complex
    Θ: float = 0.0
    nnidx: np.ndarray = field(default=None)   # (Ns, z, 2) 1-based directed bonds

    kind = KIND_TUV

    @property
    def is_complex(self) -> bool:
        return self.Type is complex

    @property
    def z(self) -> int:
        return self.nnidx.shape[1]

    @property
    def field_shape(self):
        return (self.Ns * self.z, self.Nt)


def tU_Hubbard_Para(*, Ht, Hu1, Hu2, Δt, Θrelax, Θquench, Lattice, site,
                    BatchSize, Initial, flux=0.0):
    """src/tU/model.jl:39-96."""
    site = list(site)
    Nt = round(2 * (Θrelax + Θquench) / Δt)
    Hu = _profile(Hu1, Hu2, Θrelax, Θquench, Δt, Nt)
    α = np.sqrt(Δt * Hu / 2)
    K = nnK_Matrix(Lattice, site, flux=flux)
    Ns = K.shape[0]
    HalfeK, eK, HalfeKinv, eKinv = (m.astype(np.complex128) for m in _kinetic(Ht * K, Δt))
    Pt = np.zeros((Ns, Ns // 2), dtype=np.complex128)
    if Initial == "H0":
        KK = K + 1e-5 * _stagger(Ns)
        _, V = np.linalg.eigh(KK)
        Pt[:] = V[:, : Ns // 2]
    elif Initial == "V":
        for i in range(1, Ns // 2 + 1):
            Pt[2 * i - 1, i - 1] = 1
    nodes = _nodes(Nt, BatchSize)
    return tU_Hubbard_Para_(Lattice=Lattice, site=site, Ns=Ns, Nt=Nt, K=K.astype(np.complex128),
                            BatchSize=BatchSize, Δt=Δt, γ=GAMMA.copy(), η=ETA.copy(), Pt=Pt,
                            HalfeK=HalfeK, eK=eK, HalfeKinv=HalfeKinv, eKinv=eKinv,
                            nodes=nodes, Ht=Ht, Hu1=Hu1, Hu2=Hu2, Θrelax=Θrelax,
                            Θquench=Θquench, α=α)


def _uv_blocks(Ns: int, nnidx: np.ndarray) -> np.ndarray:
    """Dense bond-rotation matrices UV[:, :, j].  src/tV/model.jl:103-110."""
    c = 2 ** 0.5 / 2
    UV = np.zeros((Ns, Ns, nnidx.shape[1]))
    for j in range(nnidx.shape[1]):
        for i in range(nnidx.shape[0]):
            x, y = nnidx[i, j] - 1
            UV[x, x, j] = UV[x, y, j] = UV[y, x, j] = -c
            UV[y, y, j] = c
    return UV


def _trial_density(K, Ns, μ, Initial, HalfeKinv):
    """Trial state of the density-channel models: top half of K's spectrum.

    src/tV/model.jl:40-76 and src/tUV/model.jl:41-77.  The staggered
    chemical potential alternates on the A/B index parity for every
    two-sublattice lattice.
    """
    Pt = np.zeros((Ns, Ns // 2))
    if Initial == "H0":
        _, V = np.linalg.eigh(K + μ * _stagger(Ns))
        Pt[:] = V[:, Ns // 2:]
    elif Initial == "V":
        for i in range(1, Ns // 2 + 1):
            Pt[2 * i - 2, i - 1] = 1
    return HalfeKinv @ Pt


def tV_Hubbard_Para(*, Ht, Hv1, Hv2, Δt, Θrelax, Θquench, Lattice, site,
                    BatchSize, Initial):
    """src/tV/model.jl:30-122."""
    site = list(site)
    K = nnK_Matrix(Lattice, site)
    Ns = K.shape[0]
    HalfeK, eK, HalfeKinv, eKinv = _kinetic(-Ht * K, Δt)
    Pt = _trial_density(K, Ns, 1e-3, Initial, HalfeKinv)
    Nt = round(2 * (Θrelax + Θquench) / Δt)
    Hv = _profile(Hv1, Hv2, Θrelax, Θquench, Δt, Nt)
    α = np.sqrt(Δt * Hv / 2)
    nnidx = nnidx_F(Lattice, site)
    return tV_Hubbard_Para_(Lattice=Lattice, site=site, Ns=Ns, Nt=Nt, K=K, BatchSize=BatchSize,
                            Δt=Δt, γ=GAMMA.copy(), η=ETA.copy(), Pt=Pt, HalfeK=HalfeK, eK=eK,
                            HalfeKinv=HalfeKinv, eKinv=eKinv, nodes=_nodes(Nt, BatchSize),
                            Ht=Ht, Hv1=Hv1, Hv2=Hv2, Θrelax=Θrelax, Θquench=Θquench, α=α,
                            nnidx=nnidx, UV=_uv_blocks(Ns, nnidx))


def tUV_Hubbard_Para(*, Ht, Hu, Hv, Lattice, site, Δt, Θ, BatchSize, Initial,
                     allow_marginal=False):
    """src/tUV/model.jl:30-118.

    ``allow_marginal=True`` relaxes the reference's strict stability assert
    ``U^2 > 4 z^2 V^2`` to ``>=`` (the decomposition stays valid at equality,
    g = U/(2z), a = V/g); the square lattices take z = 4.
    """
    site = list(site)
    if Lattice not in LATTICES:
        raise ValueError(f"Lattice: {Lattice} is not allowed !")
    K = nnK_Matrix(Lattice, site)
    Ns = K.shape[0]
    HalfeK, eK, HalfeKinv, eKinv = _kinetic(-Ht * K, Δt)
    Pt = _trial_density(K, Ns, 1e-5, Initial, HalfeKinv)
    Nt = 2 * math.ceil(Fraction(Θ) / Fraction(Δt))        # Julia 2*cld(Θ, Δt), exact
    z = 4.0 if "SQUARE" in Lattice else 3.0
    ok = Hu ** 2 >= 4 * z ** 2 * Hv ** 2 if allow_marginal else Hu ** 2 > 4 * z ** 2 * Hv ** 2
    if not ok:
        raise AssertionError("For stability, require U^2 > 4 z^2 V^2")
    Type = complex if Hu > 0 else float
    disc = max(Hu ** 2 / z ** 2 / 4 - Hv ** 2, 0.0)
    g = Hu / z / 2 + math.sqrt(disc) if Hu > 0 else Hu / z / 2 - math.sqrt(disc)
    a = 0.0 if g == 0 else Hv / g
    η = math.sqrt(abs(Δt * g)) * np.array([math.sqrt(3 - _S6), -math.sqrt(3 - _S6),
                                            math.sqrt(3 + _S6), -math.sqrt(3 + _S6)])
    tmp = nnidx_F(Lattice, site)
    nnidx = np.zeros((Ns, tmp.shape[1], 2), dtype=np.int64)
    nnidx[0::2] = tmp
    nnidx[1::2] = tmp[:, :, ::-1]
    return tUV_Hubbard_Para_(Lattice=Lattice, site=site, Ns=Ns, Nt=Nt, K=K, BatchSize=BatchSize,
                             Δt=Δt, γ=GAMMA.copy(), η=η, Pt=Pt, HalfeK=HalfeK, eK=eK,
                             HalfeKinv=HalfeKinv, eKinv=eKinv, nodes=_nodes(Nt, BatchSize),
                             Ht=Ht, U=Hu, V=Hv, a=a, Type=Type, Θ=Θ, nnidx=nnidx)


def Initial_s(model, rng) -> np.ndarray:
    """Uniform random HS field over {1,2,3,4}, Julia column-major layout.

    src/tU/GreenMatrix.jl:1-8, src/tV/GreenMatrix.jl:1-10,
    src/tUV/GreenMatrix.jl:1-8.  ``rng`` is a ``numpy.random.Generator`` or
    an integer seed (Julia's MersenneTwister stream is not reproduced).
    """
    if not isinstance(rng, np.random.Generator):
        rng = np.random.default_rng(rng)
    s = rng.integers(1, 5, size=int(np.prod(model.field_shape)), dtype=np.uint8)
    return s.reshape(model.field_shape, order="F")
