"""Handles of different lattices and models sweep concurrently (one CUDA
stream each, host calls from separate threads) with the same results as
alone: the way chains of uneven lattice sizes share the GPU."""
import threading

import numpy as np
import pytest

import cases
import dqmc_oracle as O
import philox
from kapdqmc_gb300 import Initial_s
from kapdqmc_gb300.sweep import Sweeper

pytestmark = pytest.mark.gpu


def _ref(model, s, seed, chain, sweeps):
    n = O.proposals_per_sweep(model)
    ks, us = zip(*(philox.tape(seed, chain, w, n) for w in range(sweeps)))
    return O.phy_update(model, s, sweeps, O.Tape(np.concatenate(ks), np.concatenate(us)), False)


def test_uneven_lattices_concurrently():
    models = [cases.tu_square(), cases.tv_honeycomb(), cases.tuv_honeycomb(), cases.tu_honeycomb()]
    nch, sweeps, seed = 3, 2, 99
    fields = [np.stack([Initial_s(m, 10 * k + c) for c in range(nch)]) for k, m in enumerate(models)]
    out = [None] * len(models)
    errors = []

    def work(k):
        try:
            with Sweeper(models[k], nch) as sw:
                sw.set_fields(fields[k])
                sw.set_rng(seed)
                sw.phy_update(sweeps, False)
                out[k] = sw.get_fields()
        except Exception as e:   # reported below
            errors.append(e)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(len(models))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for k, m in enumerate(models):
        for c in range(nch):
            ref = _ref(m, fields[k][c], seed, c, sweeps)
            np.testing.assert_array_equal(out[k][c], ref.s, err_msg=f"model {k} chain {c}")
