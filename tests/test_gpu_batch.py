"""Batched small instances (workload 5 generator): every instance solved by the concurrent
batch runner equals the oracle's standalone solve (det count, E_var, deterministic PT2), and
the result does not depend on the number of workers."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_matches_oracle(oracle_mod, data_dir):
    import shci_gb300
    from shci_gb300 import synthetic
    inst = []
    for i in range(6):
        path, n, ne = synthetic.batch_instance(i, data_dir)
        inst.append((path, ne, ne))
    res, used = shci_gb300._lib.batch_solve(inst, [1e-4], [], (1e-6, 1e-6, 1e-6), n_workers=3)
    res2, _ = shci_gb300._lib.batch_solve(inst, [1e-4], [], (1e-6, 1e-6, 1e-6), n_workers=0)
    for (path, nu, nd), r, r2 in zip(inst, res, res2):
        o = oracle_mod.Oracle(path, nu, nd)
        e = o.run_all_variations([1e-4], [], 5e-5)[0]
        v, _, n_pt = o.pt_dtm(1e-6, 1)
        assert r["status"] == 0
        assert r["n_dets"] == len(o.dets()[0])
        assert abs(r["energy_var"] - e) < 1e-9
        assert r["n_pt_dets"] == n_pt
        assert abs(r["correction_pt"] - v) < 1e-11
        assert r2["n_dets"] == r["n_dets"] and abs(r2["energy_var"] - r["energy_var"]) < 1e-12


def test_batch_autotuner_long_queue(data_dir):
    """A queue long enough for the autotuner (at least four times its interleaved tuning
    slices): the chosen worker count is one of its candidates, and every instance's result
    equals the same instance solved alone with two workers."""
    import os
    import shci_gb300
    from shci_gb300 import synthetic
    files = []
    for k in range(8):
        path = os.path.join(data_dir, "FCIDUMP_tune%d" % k)
        if not os.path.exists(path):
            synthetic.make(path, 12, 2 * (3 + k % 2), synthetic.BASE_SEED + 5000 + k)
        files.append((path, 3 + k % 2, 3 + k % 2))
    cpus = len(os.sched_getaffinity(0))
    cand = sorted({min(max(w, 1), 64) for w in (cpus // 4, cpus // 2, cpus)})
    n = 4 * len(cand) * 2 * cand[-1] + 16
    inst = [files[k % len(files)] for k in range(n)]
    ref, _ = shci_gb300._lib.batch_solve(files, [1e-4], [], (1e-6, 1e-6, 1e-6), n_workers=2)
    res, used = shci_gb300._lib.batch_solve(inst, [1e-4], [], (1e-6, 1e-6, 1e-6), n_workers=0)
    assert used in cand
    for k, r in enumerate(res):
        q = ref[k % len(files)]
        assert r["status"] == 0
        assert r["n_dets"] == q["n_dets"] and r["n_pt_dets"] == q["n_pt_dets"]
        assert abs(r["energy_var"] - q["energy_var"]) < 1e-12
        assert abs(r["correction_pt"] - q["correction_pt"]) < 1e-12
