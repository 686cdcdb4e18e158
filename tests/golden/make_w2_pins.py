"""Writes w2_pins.json: the oracle's results on the n = 26 synthetic workload.

Workload: synthetic FCIDUMP n = 26, 7 alpha + 7 beta electrons (shci_gb300/synthetic.py,
seed 20261203 + 2), eps_vars [5e-5] with the schedule [1e-3, 5e-4, 2e-4, 1e-4],
target_error 5e-5, variational stage only; then deterministic PT2 at eps_pt_dtm 1e-6 on the
final wavefunction (one batch).  Recorded: per-iteration det counts, symmetric nonzero counts
and energies, a SHA-256 of the final det list (alpha strings then beta strings, little-endian
u64), the final E_var, and the dtm correction with its PT det count.

The oracle (oracle/shci_oracle.cc) restates the reference's algorithm; these numbers pin it
across machines (the CPU tests re-run it) and are the targets of the GPU parity test.

Usage: python tests/golden/make_w2_pins.py
"""
import hashlib
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

EPS_VARS = [5e-5]
SCHEDULE = [1e-3, 5e-4, 2e-4, 1e-4]
TARGET_ERROR = 5e-5
EPS_PT_DTM = 1e-6


def det_digest(up, dn):
    h = hashlib.sha256()
    h.update(up.astype("<u8").tobytes())
    h.update(dn.astype("<u8").tobytes())
    return h.hexdigest()


def run(data_dir):
    from oracle.oracle import Oracle
    from shci_gb300 import synthetic
    f = synthetic.workload_fcidump(2, data_dir)
    o = Oracle(f, 7, 7)
    e = o.run_all_variations(EPS_VARS, SCHEDULE, TARGET_ERROR)
    nd, nz, en = o.iterations()
    up, dn, _ = o.dets()
    v, u, n_pt = o.pt_dtm(EPS_PT_DTM, 1)
    return {
        "workload": "synthetic n=26 7a7b C1 (seed 20261203+2)",
        "eps_vars": EPS_VARS, "schedule": SCHEDULE, "target_error": TARGET_ERROR,
        "iterations": [{"n_dets": int(a), "nnz": int(b), "energy": float(c)}
                       for a, b, c in zip(nd, nz, en)],
        "energy_var": float(e[0]),
        "n_dets": int(len(up)),
        "dets_sha256": det_digest(up, dn),
        "pt_dtm": {"eps_pt_dtm": EPS_PT_DTM, "correction": v, "n_pt_dets": int(n_pt)},
    }


if __name__ == "__main__":
    with tempfile.TemporaryDirectory() as d:
        pins = run(d)
    json.dump(pins, open(os.path.join(HERE, "w2_pins.json"), "w"), indent=1)
    print(json.dumps(pins, indent=1))
