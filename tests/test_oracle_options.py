"""CPU checks of the oracle's restatements behind the configuration options (no GPU):
<S^2> (ChemSystem::get_s2, chem_system.cc:745-798) against the expectation value of the
explicit operator S^2 = S_- S_+ + S_z (S_z + 1) built from fermion operators in numpy, and the
active-space and double-excitation switches of find_connected_dets (chem_system.cc:327-329,
345, 383-387) against the unrestricted connection lists."""
import itertools
import os

import numpy as np
import pytest


@pytest.fixture(scope="module")
def small(oracle_mod, data_dir):
    from shci_gb300 import synthetic
    path = os.path.join(data_dir, "FCIDUMP_n6")
    synthetic.make(path, 6, 5, synthetic.BASE_SEED + 7000)
    return path


def _strings(n, k):
    return [sum(1 << o for o in c) for c in itertools.combinations(range(n), k)]


def _apply(op, orb, state):
    """a^+ (op = +1) or a (op = -1) on spin-orbital orb of a 2n-bit occupation (alpha bits
    0..n-1 first, then beta), with the sign of the occupied spin-orbitals before orb.
    Returns (sign, new state) or None."""
    occ = state >> orb & 1
    if (op > 0 and occ) or (op < 0 and not occ):
        return None
    sign = -1 if bin(state & ((1 << orb) - 1)).count("1") & 1 else 1
    return sign, state ^ (1 << orb)


def _s2_explicit(n, ups, dns, coefs):
    """<psi| S_- S_+ + S_z (S_z + 1) |psi> with S_+ = sum_p a+_{p alpha} a_{p beta}."""
    dets = [u | (d << n) for u, d in zip(ups, dns)]
    index = {s: k for k, s in enumerate(dets)}
    c = np.asarray(coefs, float)

    def s_plus(vec):
        out = {}
        for s, a in vec.items():
            for p in range(n):
                r1 = _apply(-1, p + n, s)
                if r1 is None:
                    continue
                r2 = _apply(+1, p, r1[1])
                if r2 is None:
                    continue
                out[r2[1]] = out.get(r2[1], 0.0) + a * r1[0] * r2[0]
        return out

    sp = s_plus({s: c[k] for k, s in enumerate(dets)})
    nu, nd = bin(ups[0]).count("1"), bin(dns[0]).count("1")
    sz = 0.5 * (nu - nd)
    return sum(v * v for v in sp.values()) + sz * (sz + 1) * float(c @ c), index


def test_oracle_s2_equals_explicit_operator(oracle_mod, small):
    n, nu, nd = 6, 3, 2
    o = oracle_mod.Oracle(small, nu, nd)
    rng = np.random.default_rng(5)
    ups, dns = [], []
    for u in _strings(n, nu):
        for d in _strings(n, nd):
            ups.append(u)
            dns.append(d)
    # the full space (every spin-flip partner present), and a random half of it (the formula
    # skips partners that are not in the wavefunction, as the operator's projection does)
    for keep in (np.ones(len(ups), bool), rng.random(len(ups)) < 0.5):
        keep[0] = True
        u = np.array(ups, np.uint64)[keep]
        d = np.array(dns, np.uint64)[keep]
        c = rng.standard_normal(len(u))
        c /= np.linalg.norm(c)
        o.set_dets(u, d, c)
        want, _ = _s2_explicit(n, u.tolist(), d.tolist(), c)
        # S_- S_+ maps into the full space; restricted to the kept dets its expectation needs
        # the S_+ images of kept dets only, which _s2_explicit forms from the kept dets
        assert abs(o.s2() - want) < 1e-12


def test_oracle_connection_switches(oracle_mod, small):
    n, nu, nd = 6, 3, 2
    o = oracle_mod.Oracle(small, nu, nd, reorder=0)
    det = (0b000111, 0b000011)
    u0, d0, x0 = o.find_connected(det, 1e100, 1e-9)
    assert (x0 == 2).any() and (x0 == 1).any()
    o.set_has_double_excitation(False)
    u1, d1, x1 = o.find_connected(det, 1e100, 1e-9)
    assert (x1 == 1).all()
    assert set(zip(u1.tolist(), d1.tolist())) == {(a, b) for a, b, x in zip(u0.tolist(), d0.tolist(), x0.tolist()) if x == 1}
    o.set_has_double_excitation(True)
    # one active orbital per irrep (all orbitals irrep 1 here): only orbital 0 is active, so
    # every excitation whose target is above it disappears
    o.set_active_space([4])
    u2, d2, x2 = o.find_connected(det, 1e100, 1e-9)
    inactive = sum(1 << k for k in range(4, n))
    kept = {(a, b) for a, b in zip(u0.tolist(), d0.tolist())
            if not (a & ~det[0] & inactive) and not (b & ~det[1] & inactive)}
    assert set(zip(u2.tolist(), d2.tolist())) == kept and len(kept) < len(u0)
