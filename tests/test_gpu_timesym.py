"""Time-reversal symmetry (config "time_sym") on the n = 16 synthetic workload (5a5b): the
device's packed selection and Hamiltonian against the oracle's restatement of the reference's
time_sym code (solver.h:447-455, hamiltonian.h:415-598, base_system.h:86-123), the packed
variational energies against the same run without time_sym, and PT2 after unpacking."""
import json
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS = [2e-4, 1e-4]


@pytest.fixture(scope="module")
def ts(oracle_mod, w1_fcidump):
    o = oracle_mod.Oracle(w1_fcidump, 5, 5)
    o.set_time_sym(True)
    eo = o.run_all_variations(EPS, [], 5e-5)
    plain = oracle_mod.Oracle(w1_fcidump, 5, 5)
    ep = plain.run_all_variations(EPS, [], 5e-5)
    return dict(o=o, eo=eo, plain=plain, ep=ep, fcidump=w1_fcidump)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_time_sym_variation_matches_oracle(ts, prec):
    import shci_gb300 as S
    o = ts["o"]
    c = S.Context()
    c.load_fcidump(ts["fcidump"], 5, 5)
    c.set_time_sym(True)
    p = S.PREC_FP64 if prec == "fp64" else S.PREC_MIXED
    e = c.run_variation(EPS, [], 5e-5, precision=p)
    nd, nz, en = c.var_trace()
    ond, onz, oen = o.iterations()
    assert np.array_equal(nd, ond) and np.array_equal(nz, onz)
    assert np.max(np.abs(en - oen)) < 1e-8
    up, dn, _ = c.dets()
    oup, odn, _ = o.dets()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)
    assert np.all(up <= dn)
    # the packed space is the plain run's space (each open det once) with the same energies
    pup, pdn, _ = ts["plain"].dets()
    op = up != dn
    unp = set(zip(np.r_[up, dn[op]].tolist(), np.r_[dn, up[op]].tolist()))
    assert unp == set(zip(pup.tolist(), pdn.tolist()))
    assert np.max(np.abs(e - ts["ep"])) < 1e-8
    c.close()


def test_time_sym_hamiltonian_bitexact(ts):
    """The packed Hamiltonian of the final det list: element set and FP64 values equal to the
    oracle's traversal (the reference's extra passes over reversed strings)."""
    import shci_gb300 as S
    o = ts["o"]
    up, dn, coefs = o.dets()
    c = S.Context()
    c.load_fcidump(ts["fcidump"], 5, 5)
    c.set_dets(up, dn, coefs)
    c.set_time_sym(True)
    nnz, _ = c.update_hamiltonian(S.PREC_FP64)
    rp, cl, vl, diag = c.hamiltonian(nnz)
    o.clear_hamiltonian()
    onz = o.update_hamiltonian()
    orp, ocl, ovl = o.hamiltonian(onz)
    # the oracle's rows include the diagonal; compare the strict upper parts row by row
    n = len(up)
    g = {(i, int(j)): v for i in range(n) for j, v in zip(cl[rp[i]:rp[i + 1]], vl[rp[i]:rp[i + 1]])}
    r, od = {}, np.zeros(n)
    for i in range(n):
        for j, v in zip(ocl[orp[i]:orp[i + 1]], ovl[orp[i]:orp[i + 1]]):
            if j == i:
                od[i] = v
            else:
                r[(i, int(j))] = v
    assert g.keys() == r.keys()
    assert all(g[k] == r[k] for k in g)
    assert np.array_equal(diag, od)
    c.close()


def test_time_sym_pt2_after_unpack(ts):
    import shci_gb300 as S
    o = ts["o"]
    up, dn, coefs = o.dets()
    c = S.Context()
    c.load_fcidump(ts["fcidump"], 5, 5)
    c.set_dets(up, dn, coefs)
    c.set_time_sym(True)
    c.unpack_time_sym()
    o.unpack_time_sym()
    uup, udn, ucoefs = c.dets()
    oup, odn, ocoefs = o.dets()
    assert np.array_equal(uup, oup) and np.array_equal(udn, odn)
    assert np.array_equal(ucoefs, ocoefs)
    e = ts["eo"][-1]
    o.energy_var = e
    c.build_queues()
    v, _, n_pt = c.pt2_dtm(e, 1e-5, 1)
    ov, _, on_pt = o.pt_dtm(1e-5)
    assert n_pt == on_pt and abs(v - ov) < 1e-10
    c.close()


def test_cli_time_sym(tmp_path, ts):
    """The driver with "time_sym": true gives the plain run's energies (same space)."""
    import shutil
    from shci_gb300 import build
    exe = build.build_cli()
    shutil.copyfile(ts["fcidump"], tmp_path / "FCIDUMP")
    cfg = {"system": "chem", "n_up": 5, "n_dn": 5, "eps_vars": EPS, "eps_vars_schedule": [],
           "chem": {"point_group": "c1"}, "time_sym": True, "eps_pt_dtm": 1e-5,
           "eps_pt_psto": 1e-5, "eps_pt": 1e-5, "gpu": {"precision": "fp64"},
           "get_1rdm_csv": True}
    (tmp_path / "config.json").write_text(json.dumps(cfg))
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr
    res = json.load(open(tmp_path / "result.json"))
    assert abs(res["energy_var"]["1.00e-04"] - ts["ep"][-1]) < 1e-8
    lines = open(tmp_path / "1rdm.csv").read().splitlines()[1:]
    tr = sum(float(l.split(",")[2]) for l in lines if l.split(",")[0] == l.split(",")[1])
    assert abs(tr - 10.0) < 1e-8
