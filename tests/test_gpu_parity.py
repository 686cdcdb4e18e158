"""Parity of the CUDA path (through the C ABI) with the CPU oracle and the reference's
golden data.  Integer / index results must be bit-exact; FP64 matrix elements are compared
bit for bit as well (same summation order); energies within the stated tolerances."""
import numpy as np
import pytest

from conftest import C_ATOM

pytestmark = pytest.mark.gpu

SCHED_C = [2e-3, 1e-3, 5e-4, 2e-4, 1e-4]


@pytest.fixture(scope="module")
def shci():
    import shci_gb300
    return shci_gb300


def new_ctx(shci, path, n_up, n_dn, pg="C1"):
    c = shci.Context()
    c.load_fcidump(path, n_up, n_dn, pg)
    return c


@pytest.fixture(scope="module")
def c_oracle(oracle_mod):
    o = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h")
    o.run_all_variations([5e-5], SCHED_C, 5e-5)
    return o


@pytest.mark.parametrize("which", ["c_atom", "w1"])
def test_integrals_queues_hf_match_oracle(shci, oracle_mod, which, w1_fcidump):
    path, nu, nd, pg = (C_ATOM, 4, 2, "d2h") if which == "c_atom" else (w1_fcidump, 5, 5, "C1")
    o = oracle_mod.Oracle(path, nu, nd, pg)
    c = new_ctx(shci, path, nu, nd, pg)
    h1, g2, sym, order, ec = c.integrals()
    oh1, og2, osym, oorder = o.integrals()
    assert np.array_equal(h1, oh1) and np.array_equal(g2, og2)
    assert np.array_equal(sym, osym) and np.array_equal(order, oorder)
    up, dn, ehf = c.hf()
    info = o.info()
    assert (up, dn) == o.hf()
    assert ehf == info["energy_hf"]
    q = c.build_queues()
    assert q["n_hci"] == info["n_hci"] and q["n_singles"] == info["n_singles"]
    assert q["max_hci"] == info["max_hci"] and q["max_singles"] == info["max_singles"]


def test_matrix_elements_bitexact(shci, c_oracle):
    c = new_ctx(shci, C_ATOM, 4, 2, "d2h")
    up, dn, _ = c_oracle.dets()
    rng = np.random.default_rng(11)
    ui, di, uj, dj = [], [], [], []
    for i in rng.choice(len(up), 300, replace=False):
        cu, cd, nx = c_oracle.find_connected((int(up[i]), int(dn[i])), 1e100, 1e-6)
        k = rng.choice(len(cu), min(20, len(cu)), replace=False)
        ui += [up[i]] * len(k) + [up[i]]
        di += [dn[i]] * len(k) + [dn[i]]
        uj += list(cu[k]) + [up[i]]
        dj += list(cd[k]) + [dn[i]]
    got = c.h_elems(ui, di, uj, dj)
    want = np.array([c_oracle.h_elem((int(a), int(b)), (int(x), int(y)))
                     for a, b, x, y in zip(ui, di, uj, dj)])
    assert np.array_equal(got, want)


@pytest.fixture(scope="module")
def c_ham(shci, oracle_mod, c_oracle):
    """GPU and oracle Hamiltonians of the 24,087-det C-atom wavefunction (eps_var 5e-5)."""
    up, dn, coefs = c_oracle.dets()
    o = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h")
    o.set_dets(up, dn, coefs)
    onnz = o.update_hamiltonian()
    c = new_ctx(shci, C_ATOM, 4, 2, "d2h")
    c.set_dets(up, dn, coefs)
    nnz, nnz_sym = c.update_hamiltonian(shci.PREC_FP64)
    return c, o, onnz, nnz, nnz_sym, up, dn, coefs


def test_hamiltonian_connections_bitexact(c_ham, c_atom_pins):
    c, o, onnz, nnz, nnz_sym, up, dn, _ = c_ham
    n = len(up)
    assert nnz_sym == 4714387  # reference log, examples/C/out:243
    assert onnz == nnz + n
    rp, cols, vals, diag = c.hamiltonian(nnz)
    orp, ocols, ovals = o.hamiltonian(onnz)
    for i in range(n):
        a, b = int(orp[i]), int(orp[i + 1])
        oc, ov = ocols[a:b], ovals[a:b]
        assert oc[0] == i and diag[i] == ov[0]
        g0, g1 = int(rp[i]), int(rp[i + 1])
        gc, gv = cols[g0:g1], vals[g0:g1]
        so, sg = np.argsort(oc[1:], kind="stable"), np.argsort(gc, kind="stable")
        assert np.array_equal(oc[1:][so], gc[sg]), i
        assert np.array_equal(ov[1:][so], gv[sg]), i


def test_spmv_matches_oracle(c_ham):
    c, o, *_ = c_ham
    x = np.random.default_rng(5).standard_normal(c.n_dets())
    y, yo = c.hv(x), o.hv(x)
    assert np.max(np.abs(y - yo)) <= 1e-12 * np.max(np.abs(yo))


def test_mixed_spmv_fixed_point(shci, c_ham):
    """Mixed store: float-pair products with 64-bit fixed-point accumulation.  With the FP32
    residual the product matches the FP64 oracle to 1e-12 of max|y|; without it, to the FP32
    rounding of the stored values; and the result is bit-reproducible (integer sums do not
    depend on the order of the atomics)."""
    _, o, _, _, _, up, dn, coefs = c_ham
    c = new_ctx(shci, C_ATOM, 4, 2, "d2h")
    c.set_dets(up, dn, coefs)
    c.update_hamiltonian(shci.PREC_MIXED)
    rng = np.random.default_rng(7)
    for x in (rng.standard_normal(len(up)), coefs, 1e-9 * rng.standard_normal(len(up))):
        yo = o.hv(x)
        scale = np.max(np.abs(yo))
        y_res = c.hv(x, True)
        assert np.max(np.abs(y_res - yo)) <= 1e-12 * scale
        assert np.array_equal(c.hv(x, True), y_res)
        y32 = c.hv(x, False)
        assert np.max(np.abs(y32 - yo)) <= 1e-6 * scale
        assert np.array_equal(c.hv(x, False), y32)


def test_davidson_matches_oracle(c_ham):
    c, o, _, _, _, up, dn, coefs = c_ham
    e_o, vec_o, conv_o, tr_o = o.davidson(coefs, 5e-5 / 500000)
    c.set_coefs(coefs)
    e, conv, tr = c.davidson(5e-5 / 500000)
    assert conv == conv_o and len(tr) == len(tr_o)
    assert np.max(np.abs(tr - tr_o)) < 1e-10
    _, _, vec = c.dets()
    assert abs(np.dot(vec, vec_o)) / np.linalg.norm(vec) / np.linalg.norm(vec_o) > 1 - 1e-10


def test_hilbert_davidson_gpu(shci):
    import json, os
    from conftest import GOLDEN
    pins = json.load(open(os.path.join(GOLDEN, "hilbert_pins.json")))
    n = pins["n"]
    rows, cols, vals = [0], [], []
    diag = np.array([-1.0 / (2 * i + 1) for i in range(n)])
    for i in range(n):
        for j in range(i + 1, n):
            cols.append(j)
            vals.append(-1.0 / pins["gamma"] / (i + j + 1))
        rows.append(len(cols))
    init = np.zeros(n)
    init[0] = 1.0
    c = shci.Context()
    e, vec, conv = c.davidson_csr(rows, cols, vals, diag, init, pins["davidson_tol"])
    assert abs(e - pins["eigenvalue0"]) < pins["tol_value"]
    assert np.allclose(vec[:5], pins["eigenvector0_head"], atol=pins["tol_vector"])


def test_selection_matches_oracle(shci, oracle_mod):
    """Two selection steps from the same state produce identical det lists (order included)
    and identical eps_tried_prev memos."""
    o = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h")
    c = new_ctx(shci, C_ATOM, 4, 2, "d2h")
    c.build_queues()
    assert c.select(2e-3) == o.select(2e-3) == 480
    up, dn, _ = c.dets()
    oup, odn, _ = o.dets()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)
    # same coefficients in both, then a second step
    o.update_hamiltonian()
    _, vec, _, _ = o.davidson(np.r_[1.0, np.full(len(oup) - 1, 1e-16)], 5e-5 / 50)
    o.set_coefs(vec)
    c.set_coefs(vec)
    assert c.select(1e-3) == o.select(1e-3)
    up, dn, _ = c.dets()
    oup, odn, _ = o.dets()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)
    assert np.array_equal(c.eps_tried()[: len(vec)], o.eps_tried()[: len(vec)])


def test_variation_c_atom_matches_reference_log(shci, c_atom_pins):
    c = new_ctx(shci, C_ATOM, 4, 2, "d2h")
    e = c.run_variation([5e-5], SCHED_C, 5e-5)
    nd, nz, en = c.var_trace()
    ref = [it for it in c_atom_pins["iterations"] if it["eps1"] >= 5e-5]
    assert list(nd) == [it["ndets"] for it in ref]
    assert [int(z) for z, it in zip(nz, ref) if "nnz" in it] == [it["nnz"] for it in ref if "nnz" in it]
    assert abs(e[0] - c_atom_pins["energy_var"]["5.00e-05"]) < 1e-8


def test_variation_synthetic_matches_oracle(shci, oracle_mod, w1_fcidump):
    o = oracle_mod.Oracle(w1_fcidump, 5, 5)
    eo = o.run_all_variations([2e-4, 1e-4], [], 5e-5)
    c = new_ctx(shci, w1_fcidump, 5, 5)
    e = c.run_variation([2e-4, 1e-4], [], 5e-5)
    assert np.max(np.abs(e - eo)) < 1e-9
    nd, nz, _ = c.var_trace()
    ond, onz, _ = o.iterations()
    assert np.array_equal(nd, ond) and np.array_equal(nz, onz)
    up, dn, _ = c.dets()
    oup, odn, _ = o.dets()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)


@pytest.mark.parametrize("which", ["c_atom", "w1"])
def test_variation_second_rejection_matches_oracle(shci, oracle_mod, w1_fcidump, which):
    """Selection with second rejection (config "second_rejection", factor 0.2): per-iteration
    det and nonzero counts, det lists (order included) and energies equal the oracle's; the
    rejection changes the result (fewer dets than without it).  The eps_tried_prev memo is
    compared bit for bit in test_second_rejection_step_bitexact (here each side's memo follows
    its own Davidson vector, whose small coefficients differ in relative terms)."""
    if which == "c_atom":
        args, eps, sched = (C_ATOM, 4, 2, "d2h"), [1e-4], SCHED_C
    else:
        args, eps, sched = (w1_fcidump, 5, 5), [2e-4, 1e-4], []
    o = oracle_mod.Oracle(*args)
    eo = o.run_all_variations(eps, sched, 5e-5, second_rejection=True)
    c = new_ctx(shci, *args)
    c.set_second_rejection(True, 0.2)
    e = c.run_variation(eps, sched, 5e-5)
    assert np.max(np.abs(e - eo)) < 1e-9
    nd, nz, _ = c.var_trace()
    ond, onz, _ = o.iterations()
    assert np.array_equal(nd, ond) and np.array_equal(nz, onz)
    up, dn, _ = c.dets()
    oup, odn, _ = o.dets()
    assert np.array_equal(up, oup) and np.array_equal(dn, odn)
    plain = new_ctx(shci, *args)
    plain.run_variation(eps, sched, 5e-5)
    assert plain.n_dets() > c.n_dets()


def test_second_rejection_step_bitexact(shci, oracle_mod):
    """One selection step with second rejection from the same coefficients: det list and the
    eps_tried_prev memo bit for bit (memo entries from a rejected |H| included)."""
    o = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h")
    o.run_all_variations([1e-3], [2e-3], 5e-5, second_rejection=True)
    up, dn, coefs = o.dets()
    c = new_ctx(shci, C_ATOM, 4, 2, "d2h")
    c.build_queues()
    c.set_dets(up, dn, coefs)
    c.set_second_rejection(True, 0.2)
    o2 = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h")
    o2.set_dets(up, dn, coefs)
    o2.L.orc_set_second_rejection(o2.h, 1)
    assert c.select(5e-4) == o2.select(5e-4)
    gu, gd, _ = c.dets()
    ou, od, _ = o2.dets()
    assert np.array_equal(gu, ou) and np.array_equal(gd, od)
    ge, oe = c.eps_tried()[:len(up)], o2.eps_tried()[:len(up)]
    assert np.array_equal(ge, oe)
    rejected = np.abs(ge - 1.000000001 * 5e-4 / np.abs(coefs)) > 1e-12 * ge
    assert rejected.sum() > 0  # some memo entries come from a rejected |H|


def test_pt2_dtm_matches_oracle_and_reference(shci, oracle_mod, c_oracle, c_atom_pins):
    up, dn, coefs = c_oracle.dets()
    c = new_ctx(shci, C_ATOM, 4, 2, "d2h")
    c.build_queues()
    c.set_dets(up, dn, coefs)
    ev = c_oracle.energy_var
    v, u, n = c.pt2_dtm(ev, 5e-6, 1)
    vo, uo, no = c_oracle.pt_dtm(5e-6, 1)
    pin = [p for p in c_atom_pins["pt_dtm"] if p["eps_var"] == 5e-5][0]
    assert n == no == pin["n_pt_dets"]
    assert abs(v - vo) < 1e-12
    assert abs(v - pin["correction"]) < 1e-10
    v3, u3, n3 = c.pt2_dtm(ev, 5e-6, 3)
    assert n3 == n and abs(v3 - v) < 1e-12 and u3 == 0.0


def test_pt2_psto_matches_oracle_and_reference(shci, c_oracle, c_atom_pins):
    up, dn, coefs = c_oracle.dets()
    c = new_ctx(shci, C_ATOM, 4, 2, "d2h")
    c.build_queues()
    c.set_dets(up, dn, coefs)
    ev = c_oracle.energy_var
    pin = [p for p in c_atom_pins["pt_psto_first_batch"] if p["eps_var"] == 5e-5][0]
    v, u, n, b = c.pt2_psto(ev, 5e-6, pin["eps_pt_psto"], pin["n_batches"], 5e-5, 5e-8)
    vo, uo, no, bo = c_oracle.pt_psto(5e-6, pin["eps_pt_psto"], pin["n_batches"], 5e-5, 5e-8)
    assert (n, b) == (no, bo) == (pin["n_pt_dets"], 1)
    assert abs(v - vo) < 1e-13 and abs(u - uo) < 1e-13
    # the log's build had slightly different coefficients (looser Davidson tolerance): 4e-4
    # relative after the x16 extrapolation of one batch
    assert abs(v - pin["correction"]) < 1e-9
    # all 16 batches (no early stop): extrapolation ends in the exact psto sum
    v16, u16, n16, b16 = c.pt2_psto(ev, 5e-6, pin["eps_pt_psto"], 16, 0.0, 0.0)
    vo16, uo16, no16, bo16 = c_oracle.pt_psto(5e-6, pin["eps_pt_psto"], 16, 0.0, 0.0)
    assert b16 == bo16 == 16 and n16 == no16 and u16 == 0.0
    assert abs(v16 - vo16) < 1e-13
    # batch counts that are not powers of two (batch = rehash % n_batches without a division)
    for nb in (3, 7, 100):
        vb, ub, nbd, bb = c.pt2_psto(ev, 5e-6, pin["eps_pt_psto"], nb, 0.0, 0.0)
        vob, uob, nob, bob = c_oracle.pt_psto(5e-6, pin["eps_pt_psto"], nb, 0.0, 0.0)
        assert bb == bob == nb and nbd == nob
        assert abs(vb - vob) < 1e-13
        vd, ud, nd = c.pt2_dtm(ev, 5e-6, nb)
        vod, uod, nod = c_oracle.pt_dtm(5e-6, nb)
        assert nd == nod and abs(vd - vod) < 1e-13


def test_pt2_overflowing_regions_rerun_exactly(shci, c_oracle, monkeypatch):
    """With several batches each source's output region is sized by an estimate; regions far
    too small (SHCI_PT_SLOTS) make nearly every source overflow and be emitted again with an
    exact count: the results still equal the oracle's."""
    up, dn, coefs = c_oracle.dets()
    ev = c_oracle.energy_var
    monkeypatch.setenv("SHCI_PT_SLOTS", "0.3,0")
    c = new_ctx(shci, C_ATOM, 4, 2, "d2h")
    c.build_queues()
    c.set_dets(up, dn, coefs)
    for nb in (4, 7):
        v, u, n, b = c.pt2_psto(ev, 5e-6, 5e-7, nb, 0.0, 0.0)
        vo, uo, no, bo = c_oracle.pt_psto(5e-6, 5e-7, nb, 0.0, 0.0)
        assert b == bo == nb and n == no
        assert abs(v - vo) < 1e-13
        vd, ud, nd = c.pt2_dtm(ev, 5e-6, nb)
        vod, uod, nod = c_oracle.pt_dtm(5e-6, nb)
        assert nd == nod and abs(vd - vod) < 1e-13


def test_pt2_sto_matches_oracle(shci, oracle_mod, w1_fcidump):
    """Stochastic stage: the host draws the same samples as the reference's generator, so
    every iteration's estimate equals the oracle's."""
    o = oracle_mod.Oracle(w1_fcidump, 5, 5)
    o.run_all_variations([2e-4], [], 5e-5)
    up, dn, coefs = o.dets()
    c = new_ctx(shci, w1_fcidump, 5, 5)
    c.build_queues()
    c.set_dets(up, dn, coefs)
    ev = o.energy_var
    v, u, loops = c.pt2_sto(ev, 1e-6, 1e-7, 8, 3000, 347634253, 12, 5e-5, 0.0)
    vo, uo, loops_o = o.pt_sto(1e-6, 1e-7, 8, 3000, 347634253, 12, 5e-5, 0.0)
    assert len(loops) == len(loops_o) >= 6
    assert np.max(np.abs(loops - loops_o)) < 1e-14
    assert abs(v - vo) < 1e-14 and abs(u - uo) < 1e-13


@pytest.mark.parametrize("pt_mem", [1e7, 1e9])
def test_pt2_semistochastic_auto_sample_matches_oracle(shci, oracle_mod, w1_fcidump, pt_mem):
    """The reference's default stochastic stage: the sample size from the 1,000-draw pilot and
    the PT memory (1e7 B: the memory formula decides; 1e9 B: the n_var / 8 + 1 cap does), the
    top quarter of the unique-sample target deterministic, the rest sampled.  Sample size,
    deterministic count and every iteration's estimate equal the oracle's."""
    o = oracle_mod.Oracle(w1_fcidump, 5, 5)
    o.run_all_variations([2e-4, 1e-4], [], 5e-5)
    up, dn, coefs = o.dets()
    c = new_ctx(shci, w1_fcidump, 5, 5)
    c.build_queues()
    c.set_dets(up, dn, coefs)
    ev = o.energy_var
    info, info_o = {}, {}
    v, u, loops = c.pt2_sto(ev, 1e-6, 1e-8, 16, 0, 347634253, 12, 5e-5, 0.0, semisto=True,
                            pt_mem_avail=pt_mem, info=info)
    vo, uo, loops_o = o.pt_sto(1e-6, 1e-8, 16, 0, 347634253, 12, 5e-5, 0.0, semisto=True,
                               pt_mem_avail=pt_mem, info=info_o)
    assert info == info_o
    assert info["n_dtm"] > 0 and info["n_samples"] > info["n_dtm"]
    if pt_mem == 1e9:
        assert info["n_unique_target"] == len(up) // 8 + 1
    assert len(loops) == len(loops_o) >= 6
    assert np.max(np.abs(loops - loops_o)) < 1e-13
    assert abs(v - vo) < 1e-13 and abs(u - uo) < 1e-13
    # a given sample size with semisto leaves the reference's quantile heap empty: refused
    with pytest.raises(shci.ShciError):
        c.pt2_sto(ev, 1e-6, 1e-8, 16, 3000, 347634253, 12, 5e-5, 0.0, semisto=True)


def test_pt_mem_avail_formula(shci, w1_fcidump):
    """solver.h:601-611 with one process: mem_total * 0.7 - n_dets * 104 - 32 * queue entries."""
    c = new_ctx(shci, w1_fcidump, 5, 5)
    q = c.build_queues()
    n = c.n_dets()
    got = c.pt_mem_avail(64e9)
    assert got == float(int(64e9 * 0.7 - n * 104 - 32 * (q["n_hci"] + q["n_singles"])))


def test_find_connected_dets_matches_oracle(shci, c_oracle):
    """shci_find_connected_dets (BaseSystem::find_connected_dets for a batch of dets) gives
    every det's connected list in the reference's handler order, with n_excite, for windows
    that include empty ones (eps_max < eps_min), an unbounded top and eps_min = 0."""
    up, dn, coefs = c_oracle.dets()
    rng = np.random.default_rng(5)
    idx = rng.choice(len(up), 400, replace=False)
    eps_min = 10.0 ** rng.uniform(-7, -2, len(idx))
    eps_max = np.where(rng.random(len(idx)) < 0.3, 1e100, eps_min * 10.0 ** rng.uniform(-1, 3, len(idx)))
    eps_min[:5] = 0.0
    eps_max[5:10] = eps_min[5:10] * 0.5  # empty windows
    c = new_ctx(shci, C_ATOM, 4, 2, "d2h")
    c.build_queues()
    off, cu, cd, nx = c.find_connected(up[idx], dn[idx], eps_max, eps_min)
    total = 0
    for k, i in enumerate(idx):
        ou, od, onx = c_oracle.find_connected((int(up[i]), int(dn[i])), eps_max[k], eps_min[k])
        a, b = int(off[k]), int(off[k + 1])
        assert np.array_equal(cu[a:b], ou) and np.array_equal(cd[a:b], od), k
        assert np.array_equal(nx[a:b], onx.astype(np.uint8)), k
        total += len(ou)
    assert total == int(off[-1]) > 10000
    assert all(off[k + 1] == off[k] for k in range(5, 10))
    # offsets that are not the count call's are refused
    bad = off.copy()
    bad[3] += 1
    with pytest.raises(shci.ShciError):
        c._ck(c.L.shci_find_connected_dets(c.h, up[idx], dn[idx], np.ascontiguousarray(eps_max),
                                           np.ascontiguousarray(eps_min), len(idx), bad,
                                           cu.ctypes.data, cd.ctypes.data, nx.ctypes.data))


def test_mixed_precision_energy(shci, c_ham):
    c, _, _, _, _, up, dn, coefs = c_ham
    c.set_coefs(coefs)
    c.update_hamiltonian(shci.PREC_FP64)
    e64, _, _ = c.davidson(1e-10)
    c.set_coefs(coefs)
    c.update_hamiltonian(shci.PREC_MIXED)
    e32, _, _ = c.davidson(1e-10)
    ecorr = c.energy_fp64()
    assert abs(e32 - e64) < 1e-6
    assert abs(ecorr - e64) < 1e-8


def test_fp64_energy_correction_paths(shci, c_ham):
    """The FP64 energy of the Ritz vector right after Davidson reads only the residual store
    (the FP32-value part comes from Davidson's own H*v products); it equals the Rayleigh
    quotient with value + residual H*v, and any other vector (changed coefficients, a rebuilt
    matrix) takes the full product."""
    _, o, _, _, _, up, dn, coefs = c_ham
    c = new_ctx(shci, C_ATOM, 4, 2, "d2h")
    c.set_dets(up, dn, coefs)
    c.update_hamiltonian(shci.PREC_MIXED)
    c.davidson(1e-10)
    w = c.dets()[2]
    e_ritz = c.energy_fp64()
    y = c.hv(w, True)
    e_full = float(w @ y) / float(w @ w)
    assert abs(e_ritz - e_full) <= 1e-13 * abs(e_full)
    assert abs(e_ritz - float(w @ o.hv(w)) / float(w @ w)) <= 1e-12 * abs(e_full)
    assert c.energy_fp64() == e_ritz  # repeatable
    w2 = w + 1e-3 * np.random.default_rng(11).standard_normal(len(w))
    c.set_coefs(w2)
    e2 = c.energy_fp64()
    y2 = o.hv(w2)
    assert abs(e2 - float(w2 @ y2) / float(w2 @ w2)) <= 1e-12 * abs(e2)
    c.set_coefs(w)
    c.update_hamiltonian(shci.PREC_MIXED)  # same matrix, new build: full product
    assert abs(c.energy_fp64() - e_full) <= 1e-12 * abs(e_full)
