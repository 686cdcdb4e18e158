"""Edge cases of the Hamiltonian build and H*v against the oracle: the largest orbital count
(64, so orbital 63 and full-width bit strings are used), two electrons (one core entry per
det in the join), no beta electrons, a single determinant (no off-diagonal elements) and an
empty det list (rejected)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PATHS = ({}, {"SHCI_HBUILD": "join2"}, {"SHCI_HBUILD": "scan"})


def _fcidump(directory, n, n_elec, seed):
    from shci_gb300 import synthetic
    return synthetic.make(os.path.join(str(directory), "FCIDUMP_edge_n%d_s%d" % (n, seed)), n,
                          n_elec, seed)


def _random_dets(rng, n, nu, nd, count):
    """Random dets over all n orbitals plus single / double moves of them (connected pairs)."""
    def rand(k):
        return 0 if k == 0 else int(sum(1 << int(o) for o in rng.choice(n, k, replace=False)))

    def move(h):
        occ = [o for o in range(n) if h >> o & 1]
        emp = [o for o in range(n) if not h >> o & 1]
        if not occ or not emp:
            return h
        return (h & ~(1 << int(rng.choice(occ)))) | (1 << int(rng.choice(emp)))

    seen = set()
    for _ in range(count):
        u, d = rand(nu), rand(nd)
        seen.add((u, d))
        for _ in range(3):
            u2, d2 = u, d
            for _ in range(int(rng.integers(1, 3))):
                if rng.random() < 0.5 or nd == 0:
                    u2 = move(u2)
                else:
                    d2 = move(d2)
            seen.add((u2, d2))
    dets = sorted(seen)
    return (np.array([u for u, _ in dets], np.uint64), np.array([d for _, d in dets], np.uint64))


def _all_dets(n, nu, nd):
    from itertools import combinations
    ups = [sum(1 << o for o in c) for c in combinations(range(n), nu)]
    dns = [sum(1 << o for o in c) for c in combinations(range(n), nd)] if nd else [0]
    pairs = [(u, d) for u in ups for d in dns]
    return (np.array([u for u, _ in pairs], np.uint64), np.array([d for _, d in pairs], np.uint64))


def _gpu_rows(monkeypatch, path, nu, nd, up, dn, coefs, env, precision=None):
    import shci_gb300
    for k in ("SHCI_HBUILD", "SHCI_JOIN_BITS"):
        monkeypatch.delenv(k, raising=False)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    c = shci_gb300.Context()
    c.load_fcidump(path, nu, nd)
    c.set_dets(up, dn, coefs)
    nnz, _ = c.update_hamiltonian(shci_gb300.PREC_FP64 if precision is None else precision)
    rp, cols, vals, diag = c.hamiltonian(nnz)
    return c, rp, cols, vals, diag


def _check_against_oracle(monkeypatch, oracle_mod, path, nu, nd, up, dn):
    rng = np.random.default_rng(5)
    coefs = rng.standard_normal(len(up))
    coefs /= np.linalg.norm(coefs)
    o = oracle_mod.Oracle(path, nu, nd)
    o.set_dets(up, dn, coefs)
    onnz = o.update_hamiltonian()
    orp, ocols, ovals = o.hamiltonian(onnz)
    x = rng.standard_normal(len(up))
    yo = o.hv(x)
    for env in PATHS:
        c, rp, cols, vals, diag = _gpu_rows(monkeypatch, path, nu, nd, up, dn, coefs, env)
        assert int(rp[-1]) + len(up) == onnz
        for i in range(len(up)):
            a, b = int(orp[i]), int(orp[i + 1])
            assert ocols[a] == i and diag[i] == ovals[a]
            so = np.argsort(ocols[a + 1:b], kind="stable")
            g0, g1 = int(rp[i]), int(rp[i + 1])
            sg = np.argsort(cols[g0:g1], kind="stable")
            assert np.array_equal(ocols[a + 1:b][so], cols[g0:g1][sg]), (env, i)
            assert np.array_equal(ovals[a + 1:b][so], vals[g0:g1][sg]), (env, i)
        y = c.hv(x)
        assert np.max(np.abs(y - yo)) <= 1e-12 * max(1.0, np.max(np.abs(yo)))
    # mixed store: fixed-point H*v with the residual
    import shci_gb300
    c, *_ = _gpu_rows(monkeypatch, path, nu, nd, up, dn, coefs, {}, shci_gb300.PREC_MIXED)
    y = c.hv(x, True)
    assert np.max(np.abs(y - yo)) <= 1e-12 * max(1.0, np.max(np.abs(yo)))
    # Davidson from the same start vector
    e_o, _, _, _ = o.davidson(coefs, 1e-10)
    c, *_ = _gpu_rows(monkeypatch, path, nu, nd, up, dn, coefs, {})
    c.set_coefs(coefs)
    e, _, _ = c.davidson(1e-10)
    assert abs(e - e_o) < 1e-9


def test_64_orbitals(monkeypatch, oracle_mod, tmp_path):
    path = _fcidump(tmp_path, 64, 8, 20261203 + 64)
    up, dn = _random_dets(np.random.default_rng(64), 64, 4, 4, 700)
    assert int(np.bitwise_or.reduce(up | dn)) >> 63 == 1  # orbital 63 is used
    _check_against_oracle(monkeypatch, oracle_mod, path, 4, 4, up, dn)


def test_two_electrons_full_space(monkeypatch, oracle_mod, tmp_path):
    path = _fcidump(tmp_path, 10, 2, 20261203 + 2)
    up, dn = _all_dets(10, 1, 1)
    _check_against_oracle(monkeypatch, oracle_mod, path, 1, 1, up, dn)


def test_no_beta_electrons(monkeypatch, oracle_mod, tmp_path):
    path = _fcidump(tmp_path, 12, 3, 20261203 + 3)
    up, dn = _all_dets(12, 3, 0)
    _check_against_oracle(monkeypatch, oracle_mod, path, 3, 0, up, dn)


def test_single_det_and_empty_list(monkeypatch, oracle_mod, tmp_path):
    import shci_gb300
    from shci_gb300._lib import ShciError
    path = _fcidump(tmp_path, 12, 6, 20261203 + 6)
    c = shci_gb300.Context()
    c.load_fcidump(path, 3, 3)
    hu, hd, ehf = c.hf()
    for prec in (shci_gb300.PREC_FP64, shci_gb300.PREC_MIXED):
        c.set_dets(np.array([hu], np.uint64), np.array([hd], np.uint64), np.array([1.0]))
        nnz, nnz_sym = c.update_hamiltonian(prec)
        assert nnz == 0 and nnz_sym == 1
        e, _, _ = c.davidson(1e-10)
        assert abs(e - ehf) < 1e-12
        assert abs(c.hv(np.array([2.0]), prec == shci_gb300.PREC_MIXED)[0] - 2.0 * ehf) < 1e-12
    with pytest.raises(ShciError) as err:
        c.set_dets(np.array([], np.uint64), np.array([], np.uint64), np.array([]))
    assert err.value.status == 2
