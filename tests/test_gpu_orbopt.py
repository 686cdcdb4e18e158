"""Orbital-optimisation inputs from the device RDMs (src/chem/optimization.cc): the generalized
Fock matrix (:620-650), the parameter pairs (:500-522) and the gradient 2 (F_pq - F_qp)
(:565-578), against the oracle's restatement on the same wavefunction, plus two checks that
do not lean on the oracle: the energy identity E = e_core + (sum_pq D_pq h_pq + sum_m F_mm) / 2
and the gradient as the derivative of the energy under orbital rotations (central differences
of E(kappa) with the RDMs held fixed)."""
import numpy as np
import pytest

from conftest import C_ATOM

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c_atom_var(oracle_mod):
    import shci_gb300 as S
    c = S.Context()
    c.load_fcidump(C_ATOM, 4, 2, "d2h")
    e = c.run_variation([2e-4], [2e-3, 1e-3, 5e-4], 5e-5)
    o = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h")
    up, dn, coefs = c.dets()
    o.set_dets(up, dn, coefs)
    o.update_hamiltonian()
    return dict(c=c, o=o, e=e[0])


def _energy_from_rdms(g1, half, h1, g2, e_core):
    """E = e_core + sum_pq D_pq h_pq + 1/2 sum Gamma(m,r,s,q) (mq|rs) for fixed RDMs."""
    n = h1.shape[0]
    nn = n * n
    idx = np.arange(nn)
    a, b = np.meshgrid(idx, idx, indexing="ij")
    hi, lo = np.maximum(a, b), np.minimum(a, b)
    G = half[hi * (hi + 1) // 2 + lo].reshape(n, n, n, n)  # G[m, q, r, s] = Gamma(m, r, s, q)
    return e_core + np.sum(g1 * h1) + 0.5 * np.einsum("mqrs,mqrs->", G, g2)


def test_generalized_fock_and_gradient(c_atom_var):
    c, o = c_atom_var["c"], c_atom_var["o"]
    F = c.generalized_fock()
    g1, half = o.rdm1(), o.rdm2_half()
    oF = o.generalized_fock(g1, half)
    assert np.max(np.abs(F - oF)) < 1e-10
    h1, g2, sym, _, e_core = c.integrals()
    assert np.all(F[sym[:, None] != sym[None, :]] == 0.0)
    # energy identity (Helgaker 10.8.24 traced): the variational energy
    e = e_core + 0.5 * (np.sum(g1 * h1) + np.trace(F))
    assert abs(e - c_atom_var["e"]) < 1e-9
    p, q = c.orbital_parameters()
    op, oq = o.orbital_parameters()
    assert np.array_equal(p, op) and np.array_equal(q, oq) and len(p) > 0
    g = c.orbital_gradient(p, q)
    assert np.max(np.abs(g - 2 * (oF[p, q] - oF[q, p]))) < 1e-10
    assert np.max(np.abs(g)) > 1e-6  # a truncated wavefunction is not stationary in the orbitals
    # the gradient is dE/dkappa for the rotation exp(K), K_pq = -kappa, K_qp = kappa
    # (fill_rot_matrix_with_parameters, optimization.cc:524-540), RDMs fixed
    from scipy.linalg import expm
    n = h1.shape[0]
    step = 1e-4
    worst = 0.0
    for k in np.argsort(-np.abs(g))[:6]:
        es = []
        for sgn in (1, -1):
            K = np.zeros((n, n))
            K[p[k], q[k]] = -sgn * step
            K[q[k], p[k]] = sgn * step
            U = expm(K)
            h1r = U.T @ h1 @ U
            g2r = np.einsum("pi,qj,rk,sl,pqrs->ijkl", U, U, U, U, g2, optimize=True)
            es.append(_energy_from_rdms(g1, half, h1r, g2r, e_core))
        fd = (es[0] - es[1]) / (2 * step)
        worst = max(worst, abs(abs(fd) - abs(g[k])))
        assert np.sign(fd) == np.sign(g[k]) or abs(g[k]) < 1e-8
    assert worst < 1e-7


def test_generalized_fock_two_states(oracle_mod):
    """Two states: F is formed from the RDMs summed over the states (rdm.cc:222-231)."""
    import shci_gb300 as S
    c = S.Context()
    c.load_fcidump(C_ATOM, 4, 2, "d2h")
    c.set_n_states(2)
    c.run_variation([5e-4], [2e-3, 1e-3], 5e-5)
    F = c.generalized_fock()
    o = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h")
    up, dn, c0 = c.dets()
    c1 = c.state_coefs(1)
    o.set_dets(up, dn, c0)
    o.update_hamiltonian()
    g1, half = o.rdm1(), o.rdm2_half()
    o.set_coefs(c1)
    g1, half = g1 + o.rdm1(), half + o.rdm2_half()
    assert np.max(np.abs(F - o.generalized_fock(g1, half))) < 1e-10
    h1, _, _, _, e_core = c.integrals()
    es = c.state_energies()
    assert abs(2 * e_core + 0.5 * (np.sum(g1 * h1) + np.trace(F)) - es.sum()) < 1e-9
    c.close()


def test_natural_orbitals(c_atom_var):
    """Natural orbitals (optimization.cc:6-79): per irrep, the eigenvectors of the 1-RDM by
    decreasing occupation; the rotation is orthogonal, never mixes irreps, and turns the
    1-RDM diagonal with the occupations on the diagonal."""
    c = c_atom_var["c"]
    g1 = c.rdm1()
    rot, occ = c.natural_orbitals()
    n = rot.shape[0]
    _, _, sym, _, _ = c.integrals()
    assert np.max(np.abs(rot.T @ rot - np.eye(n))) < 1e-12
    assert np.all(rot[sym[:, None] != sym[None, :]] == 0.0)
    assert np.max(np.abs(rot.T @ g1 @ rot - np.diag(occ))) < 1e-10
    assert abs(occ.sum() - 6.0) < 1e-10
    for k in set(sym.tolist()):
        idx = np.where(sym == k)[0]
        want = np.sort(np.linalg.eigvalsh(g1[np.ix_(idx, idx)]))[::-1]
        assert np.max(np.abs(occ[idx] - want)) < 1e-10


def test_rotated_integrals_keep_the_spectrum(data_dir):
    """An orbital rotation is a unitary change of basis of the full CI space: the lowest
    eigenvalues of the complete-space Hamiltonian built from the rotated integrals are the
    same; rotating back restores the integrals; the rotated tables keep the 8-fold symmetry
    exactly (one value per class, as the reference's rewritten tables)."""
    import itertools
    import os
    import shci_gb300 as S
    from shci_gb300 import synthetic
    path = os.path.join(data_dir, "FCIDUMP_rot8")
    synthetic.make(path, 8, 4, synthetic.BASE_SEED + 8000)
    strs = [sum(1 << o for o in cmb) for cmb in itertools.combinations(range(8), 2)]
    up = np.array([u for u in strs for d in strs], np.uint64)
    dn = np.array([d for u in strs for d in strs], np.uint64)

    def spectrum(c):
        c.set_dets(up, dn, None)
        nnz, _ = c.update_hamiltonian(S.PREC_FP64)
        rp, cl, vl, diag = c.hamiltonian(nnz)
        m = len(diag)
        H = np.diag(diag)
        for i in range(m):
            H[i, cl[rp[i]:rp[i + 1]]] = vl[rp[i]:rp[i + 1]]
        H = np.triu(H) + np.triu(H, 1).T
        return np.linalg.eigvalsh(H)[:6]

    c = S.Context()
    c.load_fcidump(path, 2, 2)
    h0, g0, _, _, _ = c.integrals()
    e0 = spectrum(c)
    U, _ = np.linalg.qr(np.random.default_rng(3).standard_normal((8, 8)))
    c.rotate_integrals(U)
    h1, g1, _, _, _ = c.integrals()
    assert np.max(np.abs(h1 - U.T @ h0 @ U)) < 1e-12
    for perm in ((1, 0, 2, 3), (0, 1, 3, 2), (2, 3, 0, 1)):
        assert np.array_equal(g1, g1.transpose(perm))
    assert np.max(np.abs(spectrum(c) - e0)) < 1e-10
    c.rotate_integrals(U.T)
    h2, g2, _, _, _ = c.integrals()
    assert np.max(np.abs(h2 - h0)) < 1e-12 and np.max(np.abs(g2 - g0)) < 1e-12
    with pytest.raises(S.ShciError):
        c.rotate_integrals(2 * np.eye(8))
    c.close()


def _gamma_dense(half, n):
    """Gamma(P, Q, R, S) = <a+_P a+_Q a_R a_S> from the half storage (pairs P n + S, Q n + R)."""
    P, Q, R, Sx = np.meshgrid(*(np.arange(n),) * 4, indexing="ij")
    a, b = P * n + Sx, Q * n + R
    hi, lo = np.maximum(a, b), np.minimum(a, b)
    return half[hi * (hi + 1) // 2 + lo]


def test_orbital_hessian_diagonal_and_newton_step(c_atom_var):
    """Hessian diagonal (optimization.cc:605-618, 652-676) against a numpy restatement of the
    reference's formulas on the oracle's RDMs and against second differences of the energy
    with the RDMs fixed; the approximate Newton step's rotation exp(X) (:524-563) equals
    scipy's matrix exponential and lowers the fixed-RDM energy."""
    from scipy.linalg import expm
    c, o = c_atom_var["c"], c_atom_var["o"]
    h1, g2, _, _, e_core = c.integrals()
    n = h1.shape[0]
    g1, half = o.rdm1(), o.rdm2_half()
    F = o.generalized_fock(g1, half)
    G = _gamma_dense(half, n)
    p, q = c.orbital_parameters()
    hd = c.orbital_hessian_diagonal(p, q)

    def Y(a, b, cc, d):
        return (np.sum((G[a, cc, :, :] + G[a, :, cc, :]).T * g2[b, :, :, d])
                + np.sum(G[a, :, :, cc] * g2[b, d, :, :]))

    def hp(a, b, cc, d):
        v = 2 * g1[a, cc] * h1[b, d] + 2 * Y(a, b, cc, d)
        return v - (F[a, cc] + F[cc, a]) if b == d else v

    want = np.array([hp(a, b, a, b) - 2 * hp(a, b, b, a) + hp(b, a, b, a) for a, b in zip(p, q)])
    assert np.max(np.abs(hd - want)) < 1e-9 * max(1.0, np.max(np.abs(want)))
    # second differences of E(kappa) with the RDMs fixed
    step = 1e-3

    def energy(K):
        U = expm(K)
        h1r = U.T @ h1 @ U
        g2r = np.einsum("pi,qj,rk,sl,pqrs->ijkl", U, U, U, U, g2, optimize=True)
        return _energy_from_rdms(g1, half, h1r, g2r, e_core)

    e0 = energy(np.zeros((n, n)))
    for k in np.argsort(-np.abs(hd))[:3]:
        es = []
        for sgn in (1, -1):
            K = np.zeros((n, n))
            K[p[k], q[k]] = -sgn * step
            K[q[k], p[k]] = sgn * step
            es.append(energy(K))
        fd2 = (es[0] - 2 * e0 + es[1]) / step ** 2
        assert abs(fd2 - hd[k]) < 1e-4 * max(1.0, abs(hd[k]))
    # the approximate Newton step and its rotation
    g = c.orbital_gradient(p, q)
    kappa = -g / np.maximum(hd, 1e-5) * 0.1
    rot = c.orbital_rotation(p, q, kappa)
    X = np.zeros((n, n))
    X[p, q] = -kappa
    X[q, p] = kappa
    # (the reference's formula takes cos = sinc = 1 for tau^2 < 1e-10: errors ~ tau^2 / 2)
    assert np.max(np.abs(rot - expm(X))) < 1e-9
    assert np.max(np.abs(rot.T @ rot - np.eye(n))) < 1e-9
    assert energy(X) < e0
