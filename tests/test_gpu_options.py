"""Configuration options on the path, against the oracle's restatement of the reference:
<S^2> ("s2", ChemSystem::get_s2, chem_system.cc:745-798), "has_double_excitation": false
(chem_system.cc:345, hamiltonian.h:97-104, 487), the active space ("chem/active_space",
integrals.cc:295-326, chem_system.cc:327-329, 383-387), "var_sd" (solver.h:424, 446) and the
HF det options "chem/irreps" / "allow_doubly_occupy_hf" (integrals.cc:155-215)."""
import json
import shutil
import subprocess

import numpy as np
import pytest

from conftest import C_ATOM

pytestmark = pytest.mark.gpu

SCHED = [2e-3, 1e-3]


def _hamiltonian_sets(c, o, S):
    """Strict-upper element maps of the device's FP64 build and the oracle's rows."""
    nnz, _ = c.update_hamiltonian(S.PREC_FP64)
    rp, cl, vl, diag = c.hamiltonian(nnz)
    o.clear_hamiltonian()
    onz = o.update_hamiltonian()
    orp, ocl, ovl = o.hamiltonian(onz)
    n = len(rp) - 1
    g = {(i, int(j)): v for i in range(n) for j, v in zip(cl[rp[i]:rp[i + 1]], vl[rp[i]:rp[i + 1]])}
    r = {}
    for i in range(n):
        for j, v in zip(ocl[orp[i]:orp[i + 1]], ovl[orp[i]:orp[i + 1]]):
            if j != i:
                r[(i, int(j))] = v
    return g, r


def test_s2_matches_oracle_and_spin_algebra(oracle_mod):
    import shci_gb300 as S
    c = S.Context()
    c.load_fcidump(C_ATOM, 4, 2, "d2h")
    c.run_variation([5e-4], SCHED, 5e-5, precision=S.PREC_FP64)
    up, dn, coefs = c.dets()
    o = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h")
    o.set_dets(up, dn, coefs)
    s2 = c.s2()
    assert abs(s2 - o.s2()) < 1e-10
    assert abs(s2 - 2.0) < 1e-3  # the 3P ground state of carbon, Sz = 1
    # two dets related by one alpha-beta exchange of orbitals 3 and 4 (Sz = 1):
    # c_B = c_A gives the triplet S(S+1) = 2, c_B = -c_A an equal S = 1 / S = 2 mixture (4)
    a_up, a_dn = 0b1111, 0b10001
    b_up, b_dn = 0b10111, 0b1001
    for sign, want in ((1.0, 2.0), (-1.0, 4.0)):
        w = np.array([1.0, sign]) / np.sqrt(2.0)
        c.set_dets(np.array([a_up, b_up], np.uint64), np.array([a_dn, b_dn], np.uint64), w)
        assert abs(c.s2() - want) < 1e-14
        o.set_dets(np.array([a_up, b_up], np.uint64), np.array([a_dn, b_dn], np.uint64), w)
        assert abs(o.s2() - want) < 1e-14
    c.close()


def test_no_double_excitations_matches_oracle(oracle_mod):
    """Doubles off: selection and PT2 see single excitations only, the Hamiltonian leaves
    out the opposite-spin doubles (element set and FP64 values bit-exact)."""
    import shci_gb300 as S
    c = S.Context()
    c.load_fcidump(C_ATOM, 4, 2, "d2h")
    c.set_has_double_excitation(False)
    e = c.run_variation([5e-4], SCHED, 5e-5, precision=S.PREC_FP64)
    o = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h")
    o.set_has_double_excitation(False)
    eo = o.run_all_variations([5e-4], SCHED, 5e-5)
    nd, nz, en = c.var_trace()
    ond, onz, oen = o.iterations()
    assert np.array_equal(nd, ond) and np.array_equal(nz, onz)
    assert abs(e[0] - eo[0]) < 1e-9
    up, dn, coefs = c.dets()
    oup, odn, _ = o.dets()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)
    g, r = _hamiltonian_sets(c, o, S)
    assert g.keys() == r.keys() and all(g[k] == r[k] for k in g)
    # an opposite-spin double pair exists in the list but is not stored
    mixed = [(i, j) for i in range(len(up)) for j in range(i + 1, len(up))
             if up[i] != up[j] and dn[i] != dn[j]
             and bin(int(up[i]) ^ int(up[j])).count("1") == 2
             and bin(int(dn[i]) ^ int(dn[j])).count("1") == 2]
    assert mixed and not any(k in g for k in mixed)
    o.set_dets(up, dn, coefs)
    o.energy_var = e[0]
    v, _, n_pt = c.pt2_dtm(e[0], 1e-6, 1)
    ov, _, on_pt = o.pt_dtm(1e-6)
    assert n_pt == on_pt and abs(v - ov) < 1e-10
    c.close()


def test_active_space_matches_oracle(oracle_mod):
    import shci_gb300 as S
    act = [3, 2, 2, 1, 2, 1, 1, 0]  # per D2h irrep, lowest orbitals in FCIDUMP order
    c = S.Context()
    c.load_fcidump(C_ATOM, 4, 2, "d2h", reorder=0)
    c.set_active_space(act)
    mask = c.inactive_orbitals()
    _, _, sym, _, _ = c.integrals()
    want = 0
    for k in range(8):
        orbs = [i for i in range(len(sym)) if sym[i] == k + 1][:act[k]]
        hi = orbs[-1] if orbs else -1
        want |= sum(1 << i for i in range(len(sym)) if sym[i] == k + 1 and i > hi)
    assert mask == want and mask != 0
    e = c.run_variation([5e-4], SCHED, 5e-5, precision=S.PREC_FP64)
    o = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h", reorder=0)
    o.set_active_space(act)
    eo = o.run_all_variations([5e-4], SCHED, 5e-5)
    assert abs(e[0] - eo[0]) < 1e-9
    up, dn, coefs = c.dets()
    oup, odn, _ = o.dets()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)
    hu, hd, _ = c.hf()
    assert all((int(u) & ~hu & mask) == 0 and (int(d) & ~hd & mask) == 0 for u, d in zip(up, dn))
    o.set_dets(up, dn, coefs)
    o.energy_var = e[0]
    v, _, n_pt = c.pt2_dtm(e[0], 1e-6, 1)
    ov, _, on_pt = o.pt_dtm(1e-6)
    assert n_pt == on_pt and abs(v - ov) < 1e-10
    with pytest.raises(S.ShciError):
        c.set_active_space([1, 1])  # fewer entries than irreps
    c.close()


def test_var_sd_matches_oracle(oracle_mod, w1_fcidump):
    import shci_gb300 as S
    c = S.Context()
    c.load_fcidump(w1_fcidump, 5, 5)
    c.set_var_sd(True)
    e = c.run_variation([2e-4], [], 5e-5, precision=S.PREC_FP64)
    o = oracle_mod.Oracle(w1_fcidump, 5, 5)
    o.set_var_sd(True)
    eo = o.run_all_variations([2e-4], [], 5e-5)
    assert abs(e[0] - eo[0]) < 1e-9
    up, dn, _ = c.dets()
    oup, odn, _ = o.dets()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)
    plain = S.Context()
    plain.load_fcidump(w1_fcidump, 5, 5)
    plain.run_variation([2e-4], [], 5e-5, precision=S.PREC_FP64)
    assert plain.n_dets() != c.n_dets()  # every HF single and double enters at once
    c.close()
    plain.close()


def test_hf_options_match_oracle(oracle_mod):
    import shci_gb300 as S
    cases = [dict(irreps=[1, 5, 3, 2], irrep_occs_up=[1, 1, 1, 1], irrep_occs_dn=[2, 0, 0, 0]),
             dict(allow_doubly_occupy=False)]
    for kw in cases:
        c = S.Context()
        c.set_hf_options(**kw)
        c.load_fcidump(C_ATOM, 4, 2, "d2h")
        o = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h", **kw)
        assert c.hf()[:2] == o.hf()
        co, oo = c.integrals()[3], o.integrals()[3]
        assert np.array_equal(co, oo)
        if "irreps" in kw:  # an irrep-built HF det counts as explicit: no reordering
            assert np.array_equal(co, np.arange(len(co)))
        e = c.run_variation([5e-4], SCHED, 5e-5, precision=S.PREC_FP64)
        eo = o.run_all_variations([5e-4], SCHED, 5e-5)
        assert abs(e[0] - eo[0]) < 1e-9
        c.close()
    c = S.Context()
    c.set_hf_options(irreps=[7], irrep_occs_up=[4], irrep_occs_dn=[2])
    with pytest.raises(S.ShciError):
        c.load_fcidump(C_ATOM, 4, 2, "d2h")  # irrep 7 has two orbitals
    c.close()


def test_cli_options(tmp_path):
    """The driver reads the options and writes "s2" to result.json."""
    from shci_gb300 import build
    exe = build.build_cli()
    shutil.copyfile(C_ATOM, tmp_path / "FCIDUMP")
    cfg = {"system": "chem", "n_up": 4, "n_dn": 2, "eps_vars": [5e-4],
           "eps_vars_schedule": SCHED, "chem": {"point_group": "d2h"}, "var_only": True,
           "s2": True, "gpu": {"precision": "fp64"}}
    (tmp_path / "config.json").write_text(json.dumps(cfg))
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "s_squared:" in r.stdout
    res = json.load(open(tmp_path / "result.json"))
    assert abs(res["s2"] - 2.0) < 1e-3
    # the reference refuses an active space with reordered orbitals
    cfg2 = dict(cfg, chem={"point_group": "d2h", "active_space": True,
                           "irrep_active_space": [3, 2, 2, 1, 2, 1, 1, 0]})
    (tmp_path / "config.json").write_text(json.dumps(cfg2))
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode != 0 and "reorder_orbs to false" in (r.stdout + r.stderr)
    cfg2["reorder_orbs"] = False
    cfg2["has_double_excitation"] = True
    for f in tmp_path.glob("wf_eps1_*.dat"):
        f.unlink()
    (tmp_path / "config.json").write_text(json.dumps(cfg2))
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr


def test_cli_pair_contrib(tmp_path, oracle_mod, w1_fcidump):
    """"get_pair_contrib": true selects with var_sd and writes pair_contrib_<eps>.csv
    (solver.h:1227-1296), recomputed here from the written wavefunction with the oracle's
    matrix elements, in the reference's det order."""
    from shci_gb300 import build
    from test_gpu_cli import _read_wf
    exe = build.build_cli()
    shutil.copyfile(w1_fcidump, tmp_path / "FCIDUMP")
    cfg = {"system": "chem", "n_up": 5, "n_dn": 5, "eps_vars": [2e-4], "eps_vars_schedule": [],
           "chem": {"point_group": "c1"}, "var_only": True, "get_pair_contrib": True,
           "gpu": {"precision": "fp64"}}
    (tmp_path / "config.json").write_text(json.dumps(cfg))
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    res = json.load(open(tmp_path / "result.json"))
    assert res["pair_contrib"]["2.00e-04"] == "pair_contrib_2.00e-04.csv"
    lines = open(tmp_path / "pair_contrib_2.00e-04.csv").read().splitlines()
    assert lines[0] == "i,j,pair_contrib" and len(lines) == 1 + 5 * 6 // 2
    got = {(int(a), int(b)): float(v) for a, b, v in (l.split(",") for l in lines[1:])}
    w = _read_wf(tmp_path / "wf_eps1_2.00e-04.dat")
    o = oracle_mod.Oracle(tmp_path / "FCIDUMP", 5, 5)
    up, dn, coefs = w["up"], w["dn"], w["coefs"]
    hf = (int(up[0]), int(dn[0]))
    want = {}
    for d in range(1, len(up)):
        lu = [k for k in range(64) if (hf[0] & ~int(up[d])) >> k & 1]
        ld = [k for k in range(64) if (hf[1] & ~int(dn[d])) >> k & 1]
        if len(lu) + len(ld) > 2:
            continue
        if len(lu) == 2:
            i, j = lu
        elif len(lu) == 1:
            i, j = sorted([lu[0], ld[0] if ld else lu[0]])
        else:
            i, j = sorted([ld[0], ld[1] if len(ld) == 2 else ld[0]])
        h = o.h_elem(hf, (int(up[d]), int(dn[d])))
        want[(i, j)] = want.get((i, j), 0.0) + h * coefs[d] / coefs[0]
    for (i, j), v in got.items():
        x = want.get((i, j), 0.0) / (2 if i != j else 1)
        assert abs(v - x) <= 1e-13 * max(1.0, abs(x))
    assert any(abs(v) > 1e-4 for v in got.values())


def test_psto_auto_batches_matches_pilot(oracle_mod):
    """The automatic psto batch count (solver.h:772-814): the pilot's unique PT dets equal a
    recount with the oracle's connection lists, hashes and elements, and the count follows
    the reference's formula (at least 16)."""
    import math
    import shci_gb300 as S
    c = S.Context()
    c.load_fcidump(C_ATOM, 4, 2, "d2h")
    c.run_variation([1e-4], [2e-3, 1e-3, 5e-4, 2e-4], 5e-5, precision=S.PREC_FP64)
    up, dn, coefs = c.dets()
    assert len(up) > 250
    o = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h")
    o.set_dets(up, dn, coefs)
    eps = 1e-7
    var = set(zip(up.tolist(), dn.tolist()))
    pt = set()
    for i in range(50, len(up), 100):
        src = (int(up[i]), int(dn[i]))
        cu, cd, nx = o.find_connected(src, 1e100 / abs(coefs[i]), eps / abs(coefs[i]))
        for a, b, x in zip(cu.tolist(), cd.tolist(), nx.tolist()):
            if (a, b) in var or (o.L.orc_rehash(o.L.orc_det_hash(a, b)) & 127):
                continue
            if x == 1 and abs(o.h_elem(src, (a, b), 1) * coefs[i]) < eps:
                continue
            pt.add((a, b))
    for mem in (1e6, 1e15):
        nb, n_pilot = c.psto_auto_batches(eps, mem)
        assert n_pilot == len(pt) > 0
        assert nb == max(16, math.ceil(2.5 * 128 * 100 * len(pt) * 48 / mem))
    c.close()
