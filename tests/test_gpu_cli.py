"""The drop-in driver: run in a directory with config.json + FCIDUMP like the reference's
`shci`, it writes result.json with the reference's keys and prints its grep-able lines."""
import json
import os
import shutil
import subprocess

import pytest

from conftest import C_ATOM, GOLDEN

pytestmark = pytest.mark.gpu


def test_cli_c_atom_matches_reference_result(tmp_path):
    from shci_gb300 import build
    exe = build.build_cli()
    shutil.copyfile(C_ATOM, tmp_path / "FCIDUMP")
    cfg = {"system": "chem", "n_up": 4, "n_dn": 2, "eps_vars": [5e-5],
           "eps_vars_schedule": [2e-3, 1e-3, 5e-4, 2e-4, 1e-4], "chem": {"point_group": "d2h"},
           "eps_pt_dtm": 5e-6, "eps_pt_psto": 1e-7, "eps_pt": 5e-8,
           "n_dets_in_sample_pt_sto": 10000, "semisto_sto": False,
           "get_1rdm_csv": True, "2rdm": True}
    (tmp_path / "config.json").write_text(json.dumps(cfg))
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = r.stdout
    assert "Final iteration" in out and "Total energy:" in out
    res = json.load(open(tmp_path / "result.json"))
    ref = json.load(open(os.path.join(GOLDEN, "c_atom_pins.json")))
    assert res["n_elecs"] == 6
    assert abs(res["energy_hf"] - ref["energy_hf"]) < 1e-10
    assert abs(res["energy_var"]["5.00e-05"] - ref["energy_var"]["5.00e-05"]) < 1e-8
    tot = res["energy_total"]["5.00e-05"]["5.00e-08"]
    ref_tot = ref["energy_total"]["5.00e-05"]["5.00e-08"]
    # different stochastic samples (the reference used semistochastic sampling sized from
    # machine memory): agreement within the combined error bars
    assert abs(tot["value"] - ref_tot["value"]) < 5 * (tot["uncert"] + ref_tot["uncert"])
    assert res["config"]["n_up"] == 4
    lines = open(tmp_path / "1rdm.csv").read().splitlines()
    assert lines[0] == "p,r,1rdm"
    diag = sum(float(l.split(",")[2]) for l in lines[1:] if l.split(",")[0] == l.split(",")[1])
    assert abs(diag - 6.0) < 1e-8
    assert (tmp_path / "spatialRDM.txt").read_text().splitlines()[0].strip() == "22"


def test_cli_stock_stochastic_settings(tmp_path):
    """A config without n_dets_in_sample_pt_sto and with the default semisto_sto runs the
    reference's default stochastic stage (pilot-sized sample, deterministic top quarter);
    mem_total is fixed so the sample size does not depend on the machine."""
    from shci_gb300 import build
    exe = build.build_cli()
    shutil.copyfile(C_ATOM, tmp_path / "FCIDUMP")
    cfg = {"system": "chem", "n_up": 4, "n_dn": 2, "eps_vars": [5e-5],
           "eps_vars_schedule": [2e-3, 1e-3, 5e-4, 2e-4, 1e-4], "chem": {"point_group": "d2h"},
           "eps_pt_dtm": 5e-6, "eps_pt_psto": 1e-7, "eps_pt": 5e-8, "mem_total": 4e9}
    (tmp_path / "config.json").write_text(json.dumps(cfg))
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = r.stdout
    for line in ("Number of unique var dets in sample target:", "Number of dets chosen:",
                 "Number of deterministic var dets:"):
        assert line in out
    res = json.load(open(tmp_path / "result.json"))
    ref = json.load(open(os.path.join(GOLDEN, "c_atom_pins.json")))
    tot = res["energy_total"]["5.00e-05"]["5.00e-08"]
    ref_tot = ref["energy_total"]["5.00e-05"]["5.00e-08"]
    assert abs(tot["value"] - ref_tot["value"]) < 5 * (tot["uncert"] + ref_tot["uncert"])


def _read_wf(path):
    """Reads a wf_eps1_*.dat file of this build (layout documented in cli/wf_file.h)."""
    import struct

    import numpy as np
    b = open(path, "rb").read()
    assert b[:8] == b"SHCIGWF1"
    n_up, n_dn, n_states, time_sym = struct.unpack_from("<4I", b, 8)
    n, e_hf, e_var = struct.unpack_from("<Qdd", b, 24)
    o = 48
    up = np.frombuffer(b, np.uint64, n, o)
    dn = np.frombuffer(b, np.uint64, n, o + 8 * n)
    coefs = np.frombuffer(b, np.float64, n, o + 16 * n)
    assert len(b) == o + 24 * n and (n_states, time_sym) == (1, 0)
    return dict(n_up=n_up, n_dn=n_dn, e_hf=e_hf, e_var=e_var, up=up, dn=dn, coefs=coefs)


def test_cli_wavefunction_files(tmp_path):
    """wf_eps1_<eps>.dat checkpoints: written after each eps_var, loaded instead of recomputed
    on the next run (solver.h:348-397), read by the PT2 stage under skip_var; a file of another
    format is neither read nor overwritten."""
    import numpy as np
    from shci_gb300 import build
    exe = build.build_cli()
    base = {"system": "chem", "n_up": 4, "n_dn": 2, "eps_vars": [2e-4, 1e-4],
            "eps_vars_schedule": [2e-3, 1e-3, 5e-4], "chem": {"point_group": "d2h"},
            "eps_pt_dtm": 5e-6, "eps_pt_psto": 5e-6, "eps_pt": 5e-6}

    def run(d, **kw):
        d.mkdir(exist_ok=True)
        if not (d / "FCIDUMP").exists():
            shutil.copyfile(C_ATOM, d / "FCIDUMP")
        (d / "config.json").write_text(json.dumps(dict(base, **kw)))
        r = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr
        return r.stdout, json.load(open(d / "result.json"))

    a = tmp_path / "a"
    out1, res1 = run(a)  # variation + PT2, writes the files
    w = {e: _read_wf(a / ("wf_eps1_%s.dat" % e)) for e in ("2.00e-04", "1.00e-04")}
    for e, f in w.items():
        assert (f["n_up"], f["n_dn"]) == (4, 2)
        assert f["e_var"] == res1["energy_var"][e]
        assert f["e_hf"] == res1["energy_hf"]
        assert abs(np.dot(f["coefs"], f["coefs"]) - 1.0) < 1e-10
        # (thousands separators only where the en_US locale is installed)
        assert "ndets= {}".format(len(f["up"])) in out1.replace(",", "")
    # second run in the same directory: both stages loaded, nothing recomputed
    (a / "result.json").unlink()
    out2, res2 = run(a)
    assert ("Loaded {} dets from: wf_eps1_1.00e-04.dat".format(len(w["1.00e-04"]["up"]))
            in out2.replace(",", ""))
    assert "Iteration 1 " not in out2
    assert res2["energy_var"] == res1["energy_var"]
    assert res2["energy_total"] == res1["energy_total"]
    # PT2 only, from the files
    b = tmp_path / "b"
    b.mkdir()
    for e in ("2.00e-04", "1.00e-04"):
        shutil.copyfile(a / ("wf_eps1_%s.dat" % e), b / ("wf_eps1_%s.dat" % e))
    out3, res3 = run(b, skip_var=True)
    assert "Iteration" not in out3
    assert res3["energy_total"] == res1["energy_total"]
    # a file of another format is left alone and the stage is computed
    c = tmp_path / "c"
    c.mkdir()
    (c / "wf_eps1_2.00e-04.dat").write_bytes(b"\x00hps-like bytes")
    out4, res4 = run(c, eps_vars=[2e-4], var_only=True)
    assert "not a wavefunction file of this build" in out4
    assert (c / "wf_eps1_2.00e-04.dat").read_bytes() == b"\x00hps-like bytes"
    assert res4["energy_var"]["2.00e-04"] == res1["energy_var"]["2.00e-04"]


def test_cli_two_states(tmp_path):
    """n_states = 2: every state's energy_var and energy_total under the reference's keys
    (state suffix "_1", solver.h:1406-1412), the "Iteration" lines with both energies, and a
    wavefunction file holding both states; the energies equal the library's several-state run."""
    import struct

    import numpy as np
    import shci_gb300 as S
    from shci_gb300 import build
    exe = build.build_cli()
    shutil.copyfile(C_ATOM, tmp_path / "FCIDUMP")
    cfg = {"system": "chem", "n_up": 4, "n_dn": 2, "n_states": 2, "eps_vars": [2e-4],
           "eps_vars_schedule": [2e-3, 1e-3, 5e-4], "chem": {"point_group": "d2h"},
           "eps_pt_dtm": 1e-5, "eps_pt_psto": 1e-5, "eps_pt": 1e-5, "gpu": {"precision": "fp64"}}
    (tmp_path / "config.json").write_text(json.dumps(cfg))
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr
    res = json.load(open(tmp_path / "result.json"))
    e0, e1 = res["energy_var"]["2.00e-04"], res["energy_var_1"]["2.00e-04"]
    assert e0 < e1
    assert "1.00e-05" in res["energy_total"]["2.00e-04"]
    assert "1.00e-05" in res["energy_total_1"]["2.00e-04"]
    assert "(state 1)" in r.stdout
    it_lines = [l for l in r.stdout.splitlines() if l.startswith("Iteration ")]
    assert it_lines and all(len(l.split("energy=")[1].split()) == 2 for l in it_lines)
    b = (tmp_path / "wf_eps1_2.00e-04.dat").read_bytes()
    assert struct.unpack_from("<4I", b, 8)[2] == 2
    c = S.Context()
    c.load_fcidump(tmp_path / "FCIDUMP", 4, 2, "d2h")
    c.set_n_states(2)
    c.run_variation([2e-4], [2e-3, 1e-3, 5e-4], 5e-5)
    assert np.max(np.abs(c.state_energies() - [e0, e1])) < 1e-12
    c.close()


def test_integrals_cache_roundtrip(tmp_path):
    """Integrals::save_to_cache / load_from_cache (integrals.cc:17-35, 424-440): a context
    loaded from the cache holds the same prepared integrals (reordered tables, symmetries,
    orbital order, HF det) and gives the same variational energies as one that parsed the
    FCIDUMP; foreign files are neither read nor overwritten; a damaged cache is an IO error."""
    import numpy as np
    import shci_gb300 as S
    path = tmp_path / "integrals_cache.dat"
    a = S.Context()
    a.load_fcidump(C_ATOM, 4, 2, "d2h")
    assert a.save_integrals_cache(path)
    b = S.Context()
    assert b.load_integrals_cache(path, 4, 2, "d2h")
    for x, y in zip(a.integrals(), b.integrals()):
        assert np.array_equal(np.asarray(x), np.asarray(y))
    assert a.hf() == b.hf()
    ea = a.run_variation([2e-4], [2e-3, 1e-3], 5e-5, precision=S.PREC_FP64)
    eb = b.run_variation([2e-4], [2e-3, 1e-3], 5e-5, precision=S.PREC_FP64)
    # (FP64 H*v adds with atomics: equal up to the order of the additions)
    assert np.max(np.abs(ea - eb)) < 1e-12
    ua, da, _ = a.dets()
    ub, db, _ = b.dets()
    assert np.array_equal(ua, ub) and np.array_equal(da, db)
    # written for other electron counts
    with pytest.raises(S.ShciError):
        S.Context().load_integrals_cache(path, 3, 3, "d2h")
    # truncated file in this layout
    bad = tmp_path / "bad.dat"
    bad.write_bytes(path.read_bytes()[:1000])
    with pytest.raises(S.ShciError):
        S.Context().load_integrals_cache(bad, 4, 2, "d2h")
    # a file of another format (the reference's hps dump, say)
    foreign = tmp_path / "foreign.dat"
    foreign.write_bytes(b"\x01\x02not this layout" * 10)
    c = S.Context()
    assert not c.load_integrals_cache(foreign, 4, 2, "d2h")
    c.load_fcidump(C_ATOM, 4, 2, "d2h")
    assert not c.save_integrals_cache(foreign)
    assert foreign.read_bytes() == b"\x01\x02not this layout" * 10
    assert not c.load_integrals_cache(tmp_path / "missing.dat", 4, 2, "d2h")
    for x in (a, b, c):
        x.close()


def test_cli_integrals_cache(tmp_path):
    """The driver writes integrals_cache.dat after reading FCIDUMP and, with
    "load_integrals_cache": true, reads it instead of FCIDUMP (here an empty file)."""
    from shci_gb300 import build
    exe = build.build_cli()
    shutil.copyfile(C_ATOM, tmp_path / "FCIDUMP")
    cfg = {"system": "chem", "n_up": 4, "n_dn": 2, "eps_vars": [2e-4],
           "eps_vars_schedule": [2e-3, 1e-3], "chem": {"point_group": "d2h"}, "var_only": True,
           "gpu": {"precision": "fp64"}}
    (tmp_path / "config.json").write_text(json.dumps(cfg))
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "FCIDUMP cache saved to: integrals_cache.dat" in r.stdout
    e1 = json.load(open(tmp_path / "result.json"))["energy_var"]["2.00e-04"]
    (tmp_path / "FCIDUMP").write_text("")
    for f in tmp_path.glob("wf_eps1_*.dat"):
        f.unlink()
    (tmp_path / "result.json").unlink()
    cfg["load_integrals_cache"] = True
    (tmp_path / "config.json").write_text(json.dumps(cfg))
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "Loaded FCIDUMP cache from: integrals_cache.dat" in r.stdout
    assert abs(json.load(open(tmp_path / "result.json"))["energy_var"]["2.00e-04"] - e1) < 1e-12
