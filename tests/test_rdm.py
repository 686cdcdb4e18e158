"""RDMs as the adjoint of E_var (dE/dh, dE/dg).

CPU: the oracle's RDMs (restating src/chem/rdm.cc) reproduce E_var through the reference's
energy-from-RDM identity (rdm.cc:707-753), and the 1-RDM trace is the electron count.
GPU: the device RDMs equal the oracle's; wrapped in a torch.autograd.Function (test harness
only) their gradients match central finite differences of E_var in a fixed det space."""
import numpy as np
import pytest

from conftest import C_ATOM


def unpack_rdm2(half, n):
    """Dense Gamma[p,q,r,s] from the half storage of rdm.cc:233-241."""
    nn = n * n
    full = np.zeros((n, n, n, n))
    for p in range(n):
        for q in range(n):
            for r in range(n):
                for s in range(n):
                    a, b = p * n + s, q * n + r
                    if a < b:
                        a, b = b, a
                    full[p, q, r, s] = half[a * (a + 1) // 2 + b]
    return full


def energy_from_rdm(h1, g2, gamma2, n_elec, e_core):
    """rdm.cc:707-753: 1-RDM from the 2-RDM contraction, then the energy."""
    g1 = np.einsum("pkks->ps", gamma2) / (n_elec - 1.0)
    one = np.sum(g1 * h1)
    two = 0.5 * np.einsum("pqrs,psqr->", gamma2, g2)
    return e_core + one + two, g1


def test_oracle_rdm_energy_identity(oracle_mod, w1_fcidump):
    o = oracle_mod.Oracle(w1_fcidump, 5, 5)
    e = o.run_all_variations([2e-4], [], 5e-5)[0]
    up, dn, coefs = o.dets()
    o2 = oracle_mod.Oracle(w1_fcidump, 5, 5)
    o2.set_dets(up, dn, coefs)
    o2.update_hamiltonian()
    n = o2.n_orbs
    gamma2 = unpack_rdm2(o2.rdm2_half(), n)
    h1, g2, _, _ = o2.integrals()
    # E_var of the Davidson vector (coefs are normalised Ritz vectors)
    e_rdm, g1 = energy_from_rdm(h1, g2, gamma2, 10, 0.0)
    assert abs(e_rdm - e) < 1e-8
    rdm1 = o2.rdm1()
    assert abs(np.trace(rdm1) - 10.0) < 1e-8
    assert np.max(np.abs(rdm1 - g1)) < 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["c_atom", "w1"])
def test_gpu_rdms_match_oracle(oracle_mod, which, w1_fcidump):
    import shci_gb300
    if which == "c_atom":
        path, nu, nd, pg, eps, sched = C_ATOM, 4, 2, "d2h", [5e-5], [2e-3, 1e-3, 5e-4, 2e-4, 1e-4]
    else:
        path, nu, nd, pg, eps, sched = w1_fcidump, 5, 5, "C1", [2e-4], []
    o = oracle_mod.Oracle(path, nu, nd, pg)
    o.run_all_variations(eps, sched, 5e-5)
    up, dn, coefs = o.dets()
    o2 = oracle_mod.Oracle(path, nu, nd, pg)
    o2.set_dets(up, dn, coefs)
    o2.update_hamiltonian()
    c = shci_gb300.Context()
    c.load_fcidump(path, nu, nd, pg)
    c.set_dets(up, dn, coefs)
    c.update_hamiltonian(shci_gb300.PREC_FP64)
    r1, r1o = c.rdm1(), o2.rdm1()
    assert np.max(np.abs(r1 - r1o)) < 1e-12
    r2, r2o = c.rdm2_half(), o2.rdm2_half()
    assert np.max(np.abs(r2 - r2o)) < 1e-12


class _EnergyFn:
    """E_var(h1, g2) in a fixed det space on the GPU, as a torch.autograd.Function whose
    backward is the RDM adjoint (dE/dh = 1-RDM, dE/dg = Gamma / 2 at (p,s,q,r))."""

    def __init__(self, ctx, up, dn, coefs, n_up, n_dn, hf):
        import torch
        self.ctx, self.up, self.dn, self.coefs = ctx, up, dn, coefs
        self.n_up, self.n_dn, self.hf = n_up, n_dn, hf
        outer = self

        class Fn(torch.autograd.Function):
            @staticmethod
            def forward(fctx, h1, g2):
                e, r1, g = outer.solve(h1.numpy(), g2.numpy(), want_grad=True)
                fctx.save_for_backward(torch.from_numpy(r1), torch.from_numpy(g))
                return torch.tensor(e, dtype=torch.float64)

            @staticmethod
            def backward(fctx, grad):
                r1, g = fctx.saved_tensors
                return grad * r1, grad * g

        self.Fn = Fn

    def solve(self, h1, g2, want_grad=False):
        import shci_gb300
        c = self.ctx
        n = h1.shape[0]
        c.set_integrals(h1, g2, self.n_up, self.n_dn, self.hf[0], self.hf[1])
        c.set_dets(self.up, self.dn, self.coefs)
        c.update_hamiltonian(shci_gb300.PREC_FP64)
        e, conv = None, False
        for _ in range(50):
            e, conv, _ = c.davidson(1e-13)
            if conv:
                break
        assert conv
        if not want_grad:
            return e
        r1 = c.rdm1()
        gamma = unpack_rdm2(c.rdm2_half(), n)
        # E_2 = 1/2 sum Gamma(p,q,r,s) g(p,s,q,r)  ->  dE/dg[p,s,q,r] = Gamma(p,q,r,s) / 2
        dg = 0.5 * np.transpose(gamma, (0, 3, 1, 2))
        return e, r1, dg


@pytest.mark.gpu
def test_rdm_gradient_matches_finite_differences(data_dir):
    """Workload 4 (n=26, 7a7b, eps_var 5e-5): dE_var/dh and dE_var/dg from the RDMs vs
    central finite differences (step 1e-5) on 32 random symmetric integral entries."""
    import torch
    import shci_gb300
    from shci_gb300 import synthetic
    path = synthetic.workload_fcidump(4, data_dir)
    c = shci_gb300.Context()
    c.load_fcidump(path, 7, 7)
    c.run_variation([5e-5], [1e-3, 5e-4, 2e-4, 1e-4], 5e-5)
    up, dn, coefs = c.dets()
    h1, g2, _, _, _ = c.integrals()
    hf = c.hf()[:2]
    fn = _EnergyFn(c, up, dn, coefs, 7, 7, hf)
    th1 = torch.tensor(h1, requires_grad=True)
    tg2 = torch.tensor(g2, requires_grad=True)
    e = fn.Fn.apply(th1, tg2)
    e.backward()
    gh, gg = th1.grad.numpy(), tg2.grad.numpy()
    n = h1.shape[0]
    rng = np.random.default_rng(4)
    step = 1e-5
    worst = 0.0
    for k in range(32):
        dh = np.zeros_like(h1)
        dgv = np.zeros_like(g2)
        if k < 16:
            p, q = rng.integers(0, n, 2)
            dh[p, q] = dh[q, p] = 1.0
        else:
            p, q, r, s = rng.integers(0, n, 4)
            for a, b, cc, d in {(p, q, r, s), (q, p, r, s), (p, q, s, r), (q, p, s, r),
                                (r, s, p, q), (s, r, p, q), (r, s, q, p), (s, r, q, p)}:
                dgv[a, b, cc, d] = 1.0
        ep = fn.solve(h1 + step * dh, g2 + step * dgv)
        em = fn.solve(h1 - step * dh, g2 - step * dgv)
        fd = (ep - em) / (2 * step)
        an = np.sum(gh * dh) + np.sum(gg * dgv)
        worst = max(worst, abs(fd - an))
        assert abs(fd - an) < 1e-6, (k, fd, an)
    assert worst < 1e-6
