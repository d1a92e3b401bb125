"""Write the golden fixtures (``sweep_*.json``, ``scee_*.json``, ``cnn_*.json``) from the CPU oracle.

The reference ships no stored outputs (its tests run sweeps without
assertions), so these fixtures pin the oracle's own results on small models:
the initial fields, the Philox proposal stream (seed, chain 0), the
accept/reject sequence, the final fields, every measurement row, the final
Green's function and log|det(BL BR)|.  The CPU tests check that the oracle
still reproduces them; the GPU tests check the CUDA sweep against them
without running the oracle.

    python tests/golden/make_golden.py          # rewrites tests/golden/sweep_*.json
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
for p in (ROOT, ROOT / "oracle", HERE.parent):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

import cases                     # noqa: E402
import cnn_oracle as CNN         # noqa: E402
import dqmc_oracle as O          # noqa: E402
import philox                    # noqa: E402
import scee_oracle as S          # noqa: E402
from kapdqmc_gb300 import Initial_s, area_index   # noqa: E402

CASES = ["tu_square", "tu_honeycomb", "tu_quench", "tu_square90_flux", "tu_honeycomb60",
         "tv_honeycomb", "tv_honeycomb60", "tuv_honeycomb", "tuv_square", "tuv_honeycomb60"]
SEED = 1234
FIELD_SEED = 100
SWEEPS = 2


def _sensitivity(model, s, tape_k, tape_u, base) -> float:
    """Largest relative change of the measurement rows when G is perturbed by
    1e-15 relative noise before every measurement: how strongly the wraps to
    tau = Nt/2 amplify rounding for these fields."""
    cls = O._SWEEPS[model.kind]
    orig = cls.measure
    rng = np.random.default_rng(0)

    def noisy(self, lt):
        G = self.G
        self.G = G * (1 + 1e-15 * rng.standard_normal(G.shape))
        try:
            return orig(self, lt)
        finally:
            self.G = G

    cls.measure = noisy
    try:
        worst = 0.0
        for _ in range(3):
            o = np.array(O.phy_update(model, s, SWEEPS, O.Tape(tape_k, tape_u), True).obs_rows)
            worst = max(worst, float(np.abs(o - base).max() / max(1.0, np.abs(base).max())))
    finally:
        cls.measure = orig
    return worst


def make(case: str) -> dict:
    model = getattr(cases, case)()
    s = Initial_s(model, FIELD_SEED)
    n = O.proposals_per_sweep(model)
    ks, us = zip(*(philox.tape(SEED, 0, w, n) for w in range(SWEEPS)))
    tape_k, tape_u = np.concatenate(ks), np.concatenate(us)
    sw = O.phy_update(model, s, SWEEPS, O.Tape(tape_k, tape_u), True)
    sens = _sensitivity(model, s, tape_k, tape_u, np.array(sw.obs_rows))
    G = np.asarray(sw.G)
    acc = np.packbits(np.array(sw.accepts, dtype=bool)).tobytes().hex()
    return {
        "case": case, "seed": SEED, "chain": 0, "sweeps": SWEEPS, "field_seed": FIELD_SEED,
        "proposals": n * SWEEPS,
        "s": np.ravel(s, order="F").tolist(),
        "s_out": np.ravel(sw.s, order="F").tolist(),
        "n_accept": int(sum(sw.accepts)),
        "accepts_hex": acc,
        "obs": np.array(sw.obs_rows).tolist(),
        # another FP64 implementation's rows agree to within the rounding
        # the measurement wraps amplify (sensitivity x 1000), at least 1e-9
        "obs_sensitivity": sens,
        "obs_tol": max(1e-9, 1000.0 * sens),
        "G_re": np.ravel(G.real, order="F").tolist(),
        "G_im": np.ravel(G.imag, order="F").tolist() if np.iscomplexobj(G) else None,
        "log_det": O.log_det(model, sw.s)[0],
        "log_weight": O.log_weight(model, sw.s),
    }


def scee_tape(seed, sweeps, n_rep):
    """Philox stream of replica pair 0 in the coupled sweep's consumption order."""
    ks, us = [], []
    for w in range(sweeps):
        k0, u0 = philox.tape(seed, 0, w, n_rep)
        k1, u1 = philox.tape(seed, 1, w, n_rep)
        ks.append(np.stack([k0, k1], axis=1).ravel())
        us.append(np.stack([u0, u1], axis=1).ravel())
    return np.concatenate(ks), np.concatenate(us)


def make_scee() -> dict:
    """ctrl_SCEEicr on the 3x3 honeycomb t-U model: one replica pair, two sweeps."""
    m = cases.tu_honeycomb()
    L = m.site[1]
    A = area_index(m.Lattice, m.site, ([1, 1], [L // 3, L]))
    B = area_index(m.Lattice, m.site, ([1, 1], [L // 3, 2 * L // 3]))
    s1, s2 = Initial_s(m, 70), Initial_s(m, 71)
    sweeps, lam, nlam = 2, 0.5, 2
    k, u = scee_tape(SEED, sweeps, 2 * m.Ns * m.Nt)
    ref = S.SCEE(m, s1, s2, A, B, lam, nlam, O.Tape(k, u)).run(sweeps)
    G0 = np.asarray(ref.G0[0])
    return {"case": "tu_honeycomb", "seed": SEED, "sweeps": sweeps, "lam": lam, "nlam": nlam,
            "A": list(map(int, A)), "B": list(map(int, B)),
            "s": [np.ravel(s1, order="F").tolist(), np.ravel(s2, order="F").tolist()],
            "s_out": [np.ravel(ref.s[0], order="F").tolist(), np.ravel(ref.s[1], order="F").tolist()],
            "accepts_hex": np.packbits(np.array(ref.accepts, dtype=bool)).tobytes().hex(),
            "n_decisions": len(ref.accepts), "O": list(map(float, ref.O)),
            "G0_re": np.ravel(G0.real, order="F").tolist(), "G0_im": np.ravel(G0.imag, order="F").tolist()}


def make_cnn() -> dict:
    """The effective model's F and its parameter gradient on seeded fields."""
    rng = np.random.default_rng(5)
    fields = rng.integers(1, 5, size=(3, 12, 18)).astype(np.uint8)
    params = CNN.init_params(3)
    F, _ = CNN.forward(fields, params)
    dF = np.array([1.0, -0.5, 0.25])
    g = CNN.grad(fields, dF, params)
    return {"fields": fields.ravel().tolist(), "shape": list(fields.shape), "param_seed": 3,
            "dF": dF.tolist(), "F": np.asarray(F, dtype=np.float64).tolist(),
            "grad": np.asarray(g, dtype=np.float64).tolist()}


def main() -> None:
    for case in CASES:
        spec = make(case)
        path = HERE / f"sweep_{case}.json"
        path.write_text(json.dumps(spec, separators=(",", ":")) + "\n")
        print(f"{path.name}: {spec['proposals']} proposals, {spec['n_accept']} accepted, "
              f"obs tolerance {spec['obs_tol']:.1e}, {path.stat().st_size} bytes")
    for name, spec in (("scee_tu_honeycomb.json", make_scee()), ("cnn_forward_grad.json", make_cnn())):
        path = HERE / name
        path.write_text(json.dumps(spec, separators=(",", ":")) + "\n")
        print(f"{path.name}: {path.stat().st_size} bytes")


if __name__ == "__main__":
    main()
