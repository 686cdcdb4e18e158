"""CPU check (no GPU) of the orbital Hessian formulas the device kernel follows
(Optimization::hessian_diagonal / hessian_part / Y_matrix, optimization.cc:605-618, 652-676):
restated in numpy on the oracle's RDMs and generalized Fock matrix, the diagonal equals second
differences of the energy with the RDMs held fixed under orbital rotations exp(K)."""
import numpy as np
import pytest
from scipy.linalg import expm

from conftest import C_ATOM


def test_hessian_formula_equals_second_differences(oracle_mod):
    o = oracle_mod.Oracle(C_ATOM, 4, 2, "d2h")
    o.run_all_variations([5e-4], [2e-3, 1e-3], 5e-5)
    n = o.n_orbs
    h1, g2, sym, _ = o.integrals()
    info = np.zeros(6)
    o.L.orc_info(o.h, info)
    e_core = info[5]
    g1, half = o.rdm1(), o.rdm2_half()
    F = o.generalized_fock(g1, half)
    P, Q, R, Sx = np.meshgrid(*(np.arange(n),) * 4, indexing="ij")
    a, b = P * n + Sx, Q * n + R
    hi, lo = np.maximum(a, b), np.minimum(a, b)
    G = half[hi * (hi + 1) // 2 + lo]  # G[P, Q, R, S] = <a+_P a+_Q a_R a_S>

    def Y(a_, b_, c_, d_):
        return (np.sum((G[a_, c_, :, :] + G[a_, :, c_, :]).T * g2[b_, :, :, d_])
                + np.sum(G[a_, :, :, c_] * g2[b_, d_, :, :]))

    def hp(a_, b_, c_, d_):
        v = 2 * g1[a_, c_] * h1[b_, d_] + 2 * Y(a_, b_, c_, d_)
        return v - (F[a_, c_] + F[c_, a_]) if b_ == d_ else v

    idx = np.arange(n * n)
    A, B = np.meshgrid(idx, idx, indexing="ij")
    hh, ll = np.maximum(A, B), np.minimum(A, B)
    Gm = half[hh * (hh + 1) // 2 + ll].reshape(n, n, n, n)  # Gm[m, q, r, s] = Gamma(m, r, s, q)

    def energy(K):
        U = expm(K)
        h1r = U.T @ h1 @ U
        g2r = np.einsum("pi,qj,rk,sl,pqrs->ijkl", U, U, U, U, g2, optimize=True)
        return e_core + np.sum(g1 * h1r) + 0.5 * np.einsum("mqrs,mqrs->", Gm, g2r)

    e0 = energy(np.zeros((n, n)))
    pairs = [(p, q) for p in range(n) for q in range(p + 1, n) if sym[p] == sym[q]][:4]
    step = 1e-3
    for p, q in pairs:
        hd = hp(p, q, p, q) - 2 * hp(p, q, q, p) + hp(q, p, q, p)
        es = []
        for sgn in (1, -1):
            K = np.zeros((n, n))
            K[p, q] = -sgn * step
            K[q, p] = sgn * step
            es.append(energy(K))
        fd2 = (es[0] - 2 * e0 + es[1]) / step ** 2
        assert abs(fd2 - hd) < 1e-4 * max(1.0, abs(hd))
