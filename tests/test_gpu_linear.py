"""Linear-molecule (D-infinity-h) parity on the reference's Cr-dimer example (examples/Cr: 38
orbitals, 10a4b, ORBSYM in the signed linear-group labels).  The device's reordered integral
tables (Lz-screened), irreps, HF det and heat-bath queues must equal the oracle's; the
variational stage (schedule 5e-3 ... 5e-4, then eps_var = 2e-4 to convergence) must give the
oracle's det lists (order included) and per-iteration det and nonzero counts, which for the
first five iterations are also the reference log's, with energies within 1e-8 Ha of both; the
deterministic PT2 at eps_pt_dtm = 1e-5 of the device's wavefunction must count the PT dets the
oracle counts for the same wavefunction and agree within 1e-9 Ha.  (The stage's Davidson stops
at its step limit, so the two wavefunctions agree only to ~1e-8; PT2 thresholds scale with
1 / |c_i|, so PT2 is compared on one wavefunction.)"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E_TOL = 1e-8
PT_TOL = 1e-9
EPS_VAR = 2e-4
EPS_PT_DTM = 1e-5


@pytest.fixture(scope="module")
def cr(oracle_mod, cr_fcidump, cr_pins):
    p = cr_pins
    o = oracle_mod.Oracle(cr_fcidump, p["n_up"], p["n_dn"], p["point_group"])
    e = o.run_all_variations([EPS_VAR], p["eps_vars_schedule"], p["target_error"])
    return dict(o=o, e=e[0], p=p, fcidump=cr_fcidump)


def _context(cr):
    import shci_gb300 as S
    p = cr["p"]
    c = S.Context()
    c.load_fcidump(cr["fcidump"], p["n_up"], p["n_dn"], p["point_group"])
    return c


def test_cr_integrals_hf_and_queues(cr):
    o, p = cr["o"], cr["p"]
    c = _context(cr)
    h1, g2, sym, order, _ = c.integrals()
    oh1, og2, osym, oorder = o.integrals()
    assert np.array_equal(sym, osym) and np.array_equal(order, oorder)
    assert np.array_equal(h1, oh1) and np.array_equal(g2, og2)
    assert max(sym) > 2  # the example has Lz != 0 orbitals, so the screen is exercised
    u, d, e_hf = c.hf()
    assert (u, d) == o.hf()
    info = o.info()
    assert e_hf == info["energy_hf"]
    assert abs(e_hf - p["energy_hf"]) < 1e-9
    q = c.build_queues()
    assert q["n_hci"] == info["n_hci"] == p["n_hci_queue_entries"]
    assert q["max_hci"] == info["max_hci"]
    assert abs(q["max_hci"] - p["max_hci_queue_elem"]) < 1e-9
    assert q["n_singles"] == info["n_singles"] and q["max_singles"] == info["max_singles"]
    c.close()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_cr_variation_and_pt2_match_log_and_oracle(cr, prec):
    import shci_gb300 as S
    o, p = cr["o"], cr["p"]
    c = _context(cr)
    pr = S.PREC_FP64 if prec == "fp64" else S.PREC_MIXED
    e = c.run_variation([EPS_VAR], p["eps_vars_schedule"], p["target_error"], precision=pr)
    nd, nz, en = c.var_trace()
    ond, onz, oen = o.iterations()
    assert np.array_equal(nd, ond) and np.array_equal(nz, onz)
    assert np.max(np.abs(en - oen)) < E_TOL
    assert abs(e[0] - cr["e"]) < E_TOL
    for k, it in enumerate(p["iterations"]):
        assert nd[k] == it["n_dets"] and nz[k] == it["nnz"]
        assert abs(en[k] - it["energy"]) < E_TOL
    up, dn, coefs = c.dets()
    oup, odn, _ = o.dets()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)
    v, u, n_pt = c.pt2_dtm(e[0], EPS_PT_DTM, 1)
    o.set_coefs(coefs)
    o.energy_var = e[0]
    ov, ou, on_pt = o.pt_dtm(EPS_PT_DTM)
    assert n_pt == on_pt
    assert abs(v - ov) < PT_TOL and u == 0.0
    c.close()
