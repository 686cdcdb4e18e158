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



@pytest.fixture(scope="module")
def long_rows(oracle_mod, tmp_path_factory):
    """n = 26 7a7b synthetic integrals: 15,609 dets after the 1e-3 and 5e-4 selections (rows
    up to 8,597 elements) and more than 2^16 after 2e-4 and 1e-4 (tiles whose columns span
    more than 2^16 dets, so the sort's bins hold several columns)."""
    from shci_gb300 import synthetic
    path = synthetic.workload_fcidump(2, str(tmp_path_factory.mktemp("w2")))
    o = oracle_mod.Oracle(path, 7, 7)
    out = []
    for eps in (1e-3, 5e-4, 2e-4, 1e-4):
        o.run_variation_step(eps, False, 5e-5)
        if eps in (5e-4, 1e-4):
            out.append(o.dets())
    return path, out


def _raw_rows(monkeypatch, path, dets, env, precision):
    import shci_gb300
    for k in ("SHCI_HBUILD", "SHCI_JOIN_BITS", "SHCI_ROW_SORT"):
        monkeypatch.delenv(k, raising=False)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    c = shci_gb300.Context()
    c.load_fcidump(path, 7, 7)
    up, dn, coefs = dets
    c.set_dets(up, dn, coefs)
    nnz, _ = c.update_hamiltonian(precision)
    rp, cols, vals, _ = c.hamiltonian(nnz)
    return rp, cols, vals


@pytest.mark.parametrize("path", ["", "join2", "scan", "loop"])
def test_rows_in_column_order(monkeypatch, long_rows, path):
    """Every build path leaves each row in strictly increasing column order, tile by tile
    (2048 elements; rows and tail tiles of 32 or fewer elements fill one H*v chunk and are
    left as built), with the same elements per tile as the build with the pass turned off."""
    import shci_gb300
    fcidump, cases = long_rows
    # "loop": the default build, with every shared bin of the sort ranked by counting
    env = {"SHCI_ROW_SORT": "loop"} if path == "loop" else ({"SHCI_HBUILD": path} if path else {})
    for dets in cases:
        n = len(dets[0])
        for prec in (shci_gb300.PREC_FP64, shci_gb300.PREC_MIXED):
            rp, cols, vals = _raw_rows(monkeypatch, fcidump, dets, env, prec)
            rp0, cols0, vals0 = _raw_rows(monkeypatch, fcidump, dets,
                                          dict(env, SHCI_ROW_SORT="0"), prec)  # unsorted
            assert np.array_equal(rp, rp0)
            lengths = np.diff(rp.astype(np.int64))
            row = np.repeat(np.arange(n), lengths)
            pos = np.arange(len(cols)) - rp[:-1].astype(np.int64)[row]
            tile = row.astype(np.int64) * (1 << 20) + pos // 2048
            tile_len = np.minimum(2048, lengths[row] - (pos // 2048) * 2048)
            sorted_tile = tile_len > 32
            same_tile = (tile[1:] == tile[:-1]) & sorted_tile[1:]
            assert np.all(np.diff(cols.astype(np.int64))[same_tile] > 0), (n, prec)
            g0 = cols0.astype(np.int64)
            assert np.any(np.diff(g0)[same_tile] < 0)  # the switch does turn the pass off
            # the sorted build is the unsorted build's tiles in column order
            o = np.lexsort((np.where(sorted_tile, g0, 0), tile))
            assert np.array_equal(cols, cols0[o]) and np.array_equal(vals, vals0[o])
        if n < 65536:
            assert lengths.max() > 2048  # rows span several tiles
        else:
            assert lengths.max() > 2048 and n > 65536


def test_mixed_store_is_fp32_split_of_fp64(monkeypatch, c_dets):
    """The mixed store holds hi = float(H) and lo = float(H - hi) of every FP64 element:
    hi + lo, exact in FP64, equals the same split done here from the FP64 build, element by
    element."""
    import shci_gb300
    rows = {}
    for prec in (shci_gb300.PREC_FP64, shci_gb300.PREC_MIXED):
        for k in ("SHCI_HBUILD", "SHCI_JOIN_BITS", "SHCI_ROW_SORT"):
            monkeypatch.delenv(k, raising=False)
        c = shci_gb300.Context()
        c.load_fcidump(C_ATOM, 4, 2, "d2h")
        up, dn, coefs = c_dets
        c.set_dets(up, dn, coefs)
        nnz, _ = c.update_hamiltonian(prec)
        rp, cols, vals, _ = c.hamiltonian(nnz)
        row = np.repeat(np.arange(len(up)), np.diff(rp.astype(np.int64)))
        o = np.lexsort((cols, row))
        rows[prec] = (cols[o], vals[o])
    c64, v64 = rows[shci_gb300.PREC_FP64]
    cm, vm = rows[shci_gb300.PREC_MIXED]
    assert np.array_equal(c64, cm)
    hi = v64.astype(np.float32)
    lo = (v64 - hi.astype(np.float64)).astype(np.float32)
    assert np.array_equal(vm, hi.astype(np.float64) + lo.astype(np.float64))


def test_memory_budget_fallbacks_and_oom(monkeypatch, c_dets):
    """A context budget (shci_create's hbm_budget_bytes, a host-side limit) steers the build:
    from the unconstrained peak downwards it moves from the single-pass core join to the
    two-pass join, every path giving the same elements, values and (where its vectors fit)
    Davidson energy; below what any path needs, the build returns SHCI_ERR_OOM cleanly and the
    context stays usable."""
    import shci_gb300
    for k in ("SHCI_HBUILD", "SHCI_JOIN_BITS", "SHCI_ROW_SORT"):
        monkeypatch.delenv(k, raising=False)
    up, dn, coefs = c_dets

    def build(budget):
        c = shci_gb300.Context(hbm_budget=budget)
        c.load_fcidump(C_ATOM, 4, 2, "d2h")
        c.set_dets(up, dn, coefs)
        try:
            nnz, _ = c.update_hamiltonian(shci_gb300.PREC_FP64)
        except shci_gb300.ShciError as e:
            return c, None, e
        st = c.hamiltonian_stats()
        kind = "scan" if st["path"] == "group_scan" else (
            "join1" if st["one_pass"] else "join2")
        rp, cols, vals, diag = c.hamiltonian(nnz)  # packs on the host when the budget is tight
        return c, (kind, nnz, _sorted_rows(rp, cols, vals), diag), None

    c0, ref, err = build(0)
    assert err is None and ref[0] == "join1"
    peak = c0.memory_stats()[1]
    e_ref, _, _ = c0.davidson(1e-10)
    seen = {"join1"}
    oom = None
    for f in (0.9, 0.75, 0.6, 0.5, 0.4, 0.3, 0.25, 0.2, 0.15, 0.1, 0.05, 0.01):
        c, got, err = build(int(peak * f))
        if err is not None:
            assert err.status == 1, str(err)  # SHCI_ERR_OOM
            assert "budget" in str(err) or "cudaMalloc" in str(err)
            used, _, budget = c.memory_stats()
            assert used <= budget
            # the context still works after the failed build: a small det list builds
            # within the same budget and matches the reference build's leading block
            c.set_dets(up[:200], dn[:200], coefs[:200])
            nnz_small, _ = c.update_hamiltonian(shci_gb300.PREC_FP64)
            rp, cols, vals, _ = c.hamiltonian(nnz_small)
            for (ca, va), (cb, vb) in zip(_sorted_rows(rp, cols, vals), ref[2][:200]):
                keep = cb < 200
                assert np.array_equal(ca, cb[keep]) and np.array_equal(va, vb[keep])
            oom = f
            break
        kind, nnz, rows, diag = got
        seen.add(kind)
        assert nnz == ref[1] and np.array_equal(diag, ref[3])
        for (ca, va), (cb, vb) in zip(rows, ref[2]):
            assert np.array_equal(ca, cb) and np.array_equal(va, vb)
        # Davidson on the budget-built matrix, where its vectors still fit
        try:
            e, _, _ = c.davidson(1e-10)
            assert abs(e - e_ref) < 1e-12
        except shci_gb300.ShciError as ex:
            assert ex.status == 1
    assert oom is not None, "no budget small enough to fail"
    # the element store, not the join index, bounds this system: the budget moves the build
    # from one pass to two passes and then to OOM (the group scan takes over when the join
    # index cannot be built at all: 2^32 or more core entries, or SHCI_HBUILD=scan)
    assert {"join1", "join2"} <= seen, seen
