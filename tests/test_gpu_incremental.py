"""Incremental Hamiltonian updates (Hamiltonian<S>::update with n_dets_prev > 0,
src/solver/hamiltonian.h:89-93, 421-428): after a selection appends dets, the update builds
only the new rows and the old rows' new columns, as a new store segment.  The result must be
the matrix a full rebuild gives, element for element, for every consumer (export, H*v, the
FP64 energy correction, the 2-RDM), and a whole variational run must not change."""
import numpy as np
import pytest

from conftest import C_ATOM

pytestmark = pytest.mark.gpu


def _rows(c):
    nnz = c.hamiltonian_stats()["nnz"]
    rp, cols, vals, diag = c.hamiltonian(nnz)
    out = []
    for i in range(len(rp) - 1):
        a, b = int(rp[i]), int(rp[i + 1])
        o = np.argsort(cols[a:b], kind="stable")
        out.append((cols[a:b][o], vals[a:b][o]))
    return out, diag


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_incremental_update_equals_full_rebuild(monkeypatch, prec):
    import shci_gb300 as S
    monkeypatch.delenv("SHCI_HBUILD_INCREMENTAL", raising=False)
    p = S.PREC_FP64 if prec == "fp64" else S.PREC_MIXED
    a = S.Context()
    a.load_fcidump(C_ATOM, 4, 2, "d2h")
    a.build_queues()
    n_before = []
    for eps in (2e-3, 1e-3, 5e-4):  # three updates: the last two are incremental
        a.select(eps)
        n_before.append(a.n_dets())
        a.update_hamiltonian(p)
        a.davidson(1e-8)
    up, dn, coefs = a.dets()
    assert n_before[0] < n_before[1] < n_before[2] == len(up)
    b = S.Context()
    b.load_fcidump(C_ATOM, 4, 2, "d2h")
    b.set_dets(up, dn, coefs)
    b.update_hamiltonian(p)
    ra, da = _rows(a)
    rb, db = _rows(b)
    assert a.hamiltonian_stats()["nnz"] == b.hamiltonian_stats()["nnz"]
    assert np.array_equal(da, db)
    for (ca, va), (cb, vb) in zip(ra, rb):
        assert np.array_equal(ca, cb) and np.array_equal(va, vb)
    # selected rows, H*v, the FP64 energy and the 2-RDM through every segment
    rows = np.arange(0, len(up), 7, dtype=np.uint64)
    oa, ca, va = a.hamiltonian_rows(rows)
    ob, cb, vb = b.hamiltonian_rows(rows)
    assert np.array_equal(oa, ob) and np.array_equal(ca, cb) and np.array_equal(va, vb)
    x = np.random.default_rng(3).standard_normal(len(up))
    ya, yb = a.hv(x, prec == "mixed"), b.hv(x, prec == "mixed")
    # mixed: fixed-point sums do not depend on the element order; only the row abs-sum bound
    # (float sums) may round differently and move the fixed-point scale
    assert np.max(np.abs(ya - yb)) <= 1e-13 * np.max(np.abs(yb))
    a.set_coefs(coefs)
    b.set_coefs(coefs)
    ea, eb = a.energy_fp64(), b.energy_fp64()
    assert abs(ea - eb) <= 1e-12 * abs(eb)
    g_a, g_b = a.rdm2_half(), b.rdm2_half()
    assert np.max(np.abs(g_a - g_b)) < 1e-12


def test_variation_incremental_matches_full(monkeypatch, w1_fcidump):
    """A whole variational run (two eps_vars) gives the same iterations and det list, and the
    same energies to 1e-12 Ha, with incremental updates as with full rebuilds."""
    import shci_gb300 as S
    out = {}
    for inc in ("1", "0"):
        monkeypatch.setenv("SHCI_HBUILD_INCREMENTAL", inc)
        c = S.Context()
        c.load_fcidump(w1_fcidump, 5, 5)
        e = c.run_variation([2e-4, 1e-4], [5e-4], 5e-5, precision=S.PREC_MIXED)
        nd, nz, en = c.var_trace()
        up, dn, _ = c.dets()
        out[inc] = (e, nd, nz, en, up, dn)
    (e1, nd1, nz1, en1, u1, d1), (e0, nd0, nz0, en0, u0, d0) = out["1"], out["0"]
    assert np.array_equal(nd1, nd0) and np.array_equal(nz1, nz0)
    assert np.array_equal(u1, u0) and np.array_equal(d1, d0)
    assert np.max(np.abs(en1 - en0)) < 1e-12 and np.max(np.abs(e1 - e0)) < 1e-12
