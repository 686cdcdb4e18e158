"""The Hamiltonian build paths (two-hole core join in one pass with rows sized by an upper
bound, the same join in two passes with packed rows, and the group scan) produce the same
element set with bit-identical FP64 values on the 24,087-det C-atom wavefunction, also when
the join's core hash is narrowed so that most buckets merge (colliding cores)."""
import numpy as np
import pytest

from conftest import C_ATOM

pytestmark = pytest.mark.gpu


def _sorted_rows(rp, cols, vals):
    out = []
    for i in range(len(rp) - 1):
        a, b = int(rp[i]), int(rp[i + 1])
        o = np.argsort(cols[a:b], kind="stable")
        out.append((cols[a:b][o], vals[a:b][o]))
    return out


@pytest.fixture(scope="module")
def c_dets(oracle_mod):
    o = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h")
    o.run_all_variations([5e-5], [2e-3, 1e-3, 5e-4, 2e-4, 1e-4], 5e-5)
    return o.dets()


def _build(monkeypatch, dets, env):
    import shci_gb300
    for k in ("SHCI_HBUILD", "SHCI_JOIN_BITS"):
        monkeypatch.delenv(k, raising=False)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    c = shci_gb300.Context()
    c.load_fcidump(C_ATOM, 4, 2, "d2h")
    up, dn, coefs = dets
    c.set_dets(up, dn, coefs)
    nnz, nnz_sym = c.update_hamiltonian(shci_gb300.PREC_FP64)
    st = c.hamiltonian_stats()
    rp, cols, vals, diag = c.hamiltonian(nnz)
    return nnz_sym, st, _sorted_rows(rp, cols, vals), diag


def test_join_scan_and_collisions_agree(monkeypatch, c_dets):
    s_join = _build(monkeypatch, c_dets, {})
    s_scan = _build(monkeypatch, c_dets, {"SHCI_HBUILD": "scan"})
    s_two = _build(monkeypatch, c_dets, {"SHCI_HBUILD": "join2"})
    s_coll = _build(monkeypatch, c_dets, {"SHCI_JOIN_BITS": "10"})
    assert s_join[1]["path"] == "core_join" and s_coll[1]["path"] == "core_join"
    assert s_two[1]["path"] == "core_join"
    assert s_scan[1]["path"] == "group_scan"
    n = len(c_dets[0])
    assert s_join[1]["core_entries"] == n * 15  # C(6, 2) electron pairs per det
    # 1024 buckets for ~361k entries: nearly all cores collide, far more candidates
    assert s_coll[1]["candidates"] > 20 * s_join[1]["candidates"]
    for other in (s_scan, s_two, s_coll):
        assert other[0] == s_join[0] == 4714387  # reference log, examples/C/out:243
        assert np.array_equal(other[3], s_join[3])
        for (ca, va), (cb, vb) in zip(s_join[2], other[2]):
            assert np.array_equal(ca, cb) and np.array_equal(va, vb)
