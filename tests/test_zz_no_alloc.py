"""shci_hamiltonian_elems_noalloc (the entry point for callers that cannot allocate device
memory) gives exactly the results of shci_hamiltonian_elems, on two calls in a row, and
rejects requests beyond its fixed scratch size.  Kept in its own file so it runs last."""
import numpy as np
import pytest

from conftest import C_ATOM

pytestmark = pytest.mark.gpu

N_ORB, N_UP, N_DN = 22, 4, 2


def _random_pairs(rng, n):
    """Det pairs of the C atom (22 orbitals, 4 up / 2 dn): random dets and, for each, a det
    0 to 3 random single-electron moves away (degrees 0, 1, 2 and > 2 all occur)."""
    def rand_half(k):
        return int(sum(1 << int(o) for o in rng.choice(N_ORB, k, replace=False)))

    def move(h):
        occ = [o for o in range(N_ORB) if h >> o & 1]
        emp = [o for o in range(N_ORB) if not h >> o & 1]
        return (h & ~(1 << int(rng.choice(occ)))) | (1 << int(rng.choice(emp)))

    ui, di, uj, dj = [], [], [], []
    for _ in range(n):
        u, d = rand_half(N_UP), rand_half(N_DN)
        u2, d2 = u, d
        for _ in range(int(rng.integers(0, 4))):
            if rng.random() < 0.5:
                u2 = move(u2)
            else:
                d2 = move(d2)
        ui.append(u)
        di.append(d)
        uj.append(u2)
        dj.append(d2)
    return [np.array(x, np.uint64) for x in (ui, di, uj, dj)]


def test_noalloc_matches_existing_entry_point_twice():
    import shci_gb300
    ctx = shci_gb300.Context()
    ctx.load_fcidump(C_ATOM, N_UP, N_DN, "d2h")
    rng = np.random.default_rng(2024)
    # two calls in a row; the second is smaller, so stale scratch from the first lies beyond
    # its range and must not leak into its results
    for n in (5000, 1200):
        ui, di, uj, dj = _random_pairs(rng, n)
        want = ctx.h_elems(ui, di, uj, dj)
        got = ctx.h_elems_noalloc(ui, di, uj, dj)
        assert np.array_equal(got, want)
        assert np.count_nonzero(want) > n // 4  # the batch exercises non-zero elements


def test_noalloc_full_size_and_allocates_nothing():
    """A call at exactly the 65,536-pair limit (every slot of the scratch array and the start
    of its result region in use) matches the allocating entry point, and after a warm-up
    call the device's free memory is the same before and after a call."""
    import torch
    import shci_gb300
    ctx = shci_gb300.Context()
    ctx.load_fcidump(C_ATOM, N_UP, N_DN, "d2h")
    rng = np.random.default_rng(77)
    ui, di, uj, dj = _random_pairs(rng, 65536)
    want = ctx.h_elems(ui, di, uj, dj)
    ctx.h_elems_noalloc(ui[:10], di[:10], uj[:10], dj[:10])  # warm-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    got = ctx.h_elems_noalloc(ui, di, uj, dj)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert np.array_equal(got, want)
    assert free1 == free0


def test_noalloc_rejects_oversized_requests():
    import shci_gb300
    from shci_gb300._lib import ShciError
    ctx = shci_gb300.Context()
    ctx.load_fcidump(C_ATOM, N_UP, N_DN, "d2h")
    n = 65537
    z = np.full(n, 0xF, np.uint64)
    with pytest.raises(ShciError) as e:
        ctx.h_elems_noalloc(z, z, z, z)
    assert e.value.status == 2 and "65536" in str(e.value)
