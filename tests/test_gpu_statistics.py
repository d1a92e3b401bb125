"""Statistical agreement of the mixed-precision and self-learning sweeps with
the plain FP64 sweep at the configured lattice sizes, and of the Rényi-2
replica estimator with the exact Fock-space sum.

Same-law comparison (mixed vs FP64).  The mixed sweep implements the FP64
sweep's Markov kernel up to rounding.  Started from the same fields with
independent random streams, chain c of either arm has the same
distribution after every sweep, whether or not the chains have reached
equilibrium, so the per-chain averages of any observable over the same
sweeps have the same expectation.  The test forms the paired differences
d_c = mean_mixed(c) - mean_fp64(c) over the chains and asserts
|mean(d)| / se(d) < Z_MAX for the energy, the double occupancy, the
corrected AF spin structure factor and, for the t-UV replica pairs, the
Rényi-2 estimator e^-S2 = <|det g_A|^2> (Ek: src/tU/phy_update.jl:184;
Eu: :186-190; structure factors: :194-235 with every term; Grover
determinant: src/public/GF.jl:101-109 and src/tU/SCEE.jl:264-276).  The
z-scores are printed.

Equilibrium comparison (self-learning cluster moves).  The cluster moves
change the Markov kernel, not its stationary distribution (each move is
accepted with the exact determinant ratio), so mixed chains with and without
them agree after burn-in; the chain means are independent samples.
"""
import math

import numpy as np
import pytest

import cases
import fock_oracle as F
from kapdqmc_gb300 import Initial_s, area_index, slmc
from kapdqmc_gb300.sweep import Sweeper

pytestmark = pytest.mark.gpu

Z_MAX = 3.5        # per observable; 12 z-scores at this bound fail by chance ~0.6 % of the time


def _sweeps(model, prec, fields, seed, sweeps, middle_index=None, slmc_args=None, burn=0):
    """(chains, sweeps, n_obs) rows after `burn` unrecorded sweeps, and
    (sweeps, pairs) |det g_A|^2 of the chain pairs at tau = Nt/2 when
    middle_index is given."""
    dets = []
    with Sweeper(model, len(fields)) as sw:
        sw.set_precision(prec)
        sw.set_measure_full(True)
        sw.set_fields(fields)
        sw.set_rng(seed)
        if slmc_args is not None:
            sw.slmc_enable(*slmc_args)
        sw.init()
        if burn:
            sw.sweep(burn, record=0)
        if middle_index is not None:
            sw.keep_middle_green(True)
        for _ in range(sweeps):
            sw.sweep(1, record=2)
            if middle_index is not None:
                sw.synchronize()
                dets.append(np.abs(sw.grover_det_middle(middle_index)) ** 2)
        sw.synchronize()
        obs = sw.get_obs(sweeps)
    return obs, (np.array(dets) if dets else None)


def _paired_z(a, b):
    d = a - b
    se = d.std(ddof=1) / math.sqrt(len(d))
    return float(d.mean() / se) if se > 0 else 0.0


CONFIGS = {
    # name: (columns, chains, sweeps)
    "c3": ({"Ek": 0, "Eu": 1, "S_AF": 8}, 128, 6),
    "c5": ({"Ek": 0, "Eu": 1, "S_AF": 8}, 128, 6),
    "c4": ({"Ek": 0, "Eu": 1, "Ev": 2, "S_AF": 9}, 256, 6),
}


@pytest.mark.parametrize("name", ["c3", "c4", "c5"])
def test_mixed_matches_fp64_in_law_at_config_size(name):
    model = getattr(cases, name)()
    cols, nch, sweeps = CONFIGS[name]
    fields = np.stack([Initial_s(model, 6100 + c) for c in range(nch)])
    index = None
    if name == "c4":   # replica pairs (2c, 2c+1), region A = the left half
        index = area_index("SQUARE45", list(model.site), ((1, 1), (model.site[0], model.site[1])))
    mx, dmx = _sweeps(model, "mixed", fields, 11, sweeps, index)
    fp, dfp = _sweeps(model, "fp64", fields, 12, sweeps, index)
    z = {k: _paired_z(mx[:, :, q].mean(axis=1), fp[:, :, q].mean(axis=1)) for k, q in cols.items()}
    if index is not None:
        z["exp_minus_S2"] = _paired_z(dmx.mean(axis=0), dfp.mean(axis=0))
    print(name, "mixed - fp64 z-scores:", {k: round(v, 2) for k, v in z.items()})
    assert all(abs(v) < Z_MAX for v in z.values()), z
    # the structure factor is measured, not identically zero
    assert abs(fp[:, :, cols["S_AF"]].mean()) > 1e-3


def test_cluster_moves_match_local_sweep_at_config_size():
    """t-U 9x9 honeycomb (N = 162), mixed precision: local updates only
    against local updates plus one 32-site cluster move per slice, after
    burn-in; Ek, Eu and the corrected SDW0 agree."""
    model = cases.c5()
    nch, burn, sweeps = 128, 20, 12
    params = (slmc.init_params(3) * 0.05).astype(np.float32)
    res = {}
    for arm, args, seed in (("local", None, 21), ("slmc", (params, 1, 32, 64), 22)):
        fields = np.stack([Initial_s(model, 7000 + 1000 * (arm == "slmc") + c) for c in range(nch)])
        obs, _ = _sweeps(model, "mixed", fields, seed, sweeps, slmc_args=args, burn=burn)
        res[arm] = obs.mean(axis=1)
    z = {}
    for k, q in {"Ek": 0, "Eu": 1, "S_AF": 8}.items():
        a, b = res["slmc"][:, q], res["local"][:, q]
        z[k] = (a.mean() - b.mean()) / math.hypot(a.std(ddof=1) / math.sqrt(nch), b.std(ddof=1) / math.sqrt(nch))
    print("slmc - local z-scores:", {k: round(v, 2) for k, v in z.items()})
    assert all(abs(v) < Z_MAX for v in z.values()), z


def test_renyi2_replicas_match_exact_sum():
    """e^-S2 = <|det(2 G1 G2 - G1 - G2 + I)_A|^2> over 256 independent
    replica pairs of the GPU sweep on the 8-site honeycomb lattice, region A
    = 4 sites, against the exact Tr(rho_A^2) of the sweep's state."""
    model = cases.tu_hc8()
    A = [1, 2, 3, 4]                                  # 1-based sites
    exact = F.tu_renyi2(model, [a - 1 for a in A]).real
    for prec in ("fp64", "mixed"):
        fields = np.stack([Initial_s(model, 8000 + c) for c in range(512)])
        _, dets = _sweeps(model, prec, fields, 31, 120, middle_index=A, burn=20)
        pair_means = dets.mean(axis=0)
        mu, se = pair_means.mean(), pair_means.std(ddof=1) / math.sqrt(len(pair_means))
        print(prec, "e^-S2", mu, "+-", se, "exact", exact)
        assert abs(mu - exact) < 5 * se, (prec, mu, se, exact)
        assert se < 0.1 * exact
