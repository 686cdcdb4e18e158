"""Synthetic FCIDUMP generator (seeded) for the benchmark workloads.

Integrals (no symmetry, E_core = 0):
  h_pq   = delta_pq * (-2 + 4 p / n) + 0.05 * (A + A^T)_pq / 2,  A ~ N(0, 1)
  g_pqrs = sum_{L < 2n} B^L_pq B^L_rs,  B^L symmetric with
           B^L_pq ~ N(0, sigma = 0.3 / sqrt(2 n)) * exp(-|p - q| / 4)
Entries are written 8-fold unique (p >= q, r >= s, pq >= rs), 1-based, |v| < 1e-9 dropped, in
the FCIDUMP layout the reference reads (src/chem/integrals.cc:37-114).

Draw order with numpy.random.default_rng(seed): A (n x n), then for L = 0 .. 2n-1 one
n x n standard-normal matrix whose upper triangle (with diagonal) is mirrored.
Seeds: 20261203 + k for workload k (k = 1..5); batch instance i uses 20261203 + 1000 + i.
"""
import os

import numpy as np

BASE_SEED = 20261203

# Workloads (n orbitals, electrons per spin) with their seeds.
WORKLOADS = {
    1: dict(n=16, n_up=5, n_dn=5),
    2: dict(n=26, n_up=7, n_dn=7),
    3: dict(n=40, n_up=10, n_dn=10),
    4: dict(n=26, n_up=7, n_dn=7),
}


def integrals(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n))
    h = np.diag(-2.0 + 4.0 * np.arange(n) / n) + 0.05 * (A + A.T) / 2.0
    sigma = 0.3 / np.sqrt(2.0 * n)
    p = np.arange(n)
    decay = np.exp(-np.abs(p[:, None] - p[None, :]) / 4.0)
    B = np.empty((2 * n, n, n))
    for L in range(2 * n):
        U = rng.standard_normal((n, n))
        S = np.triu(U) + np.triu(U, 1).T
        B[L] = S * sigma * decay
    g = np.einsum("lpq,lrs->pqrs", B, B)
    return h, g


def write_fcidump(path, h, g, n_elec, e_core=0.0):
    n = h.shape[0]
    lines = [" &FCI NORB=%d,NELEC=%d,MS2=0," % (n, n_elec),
             "  ORBSYM=" + ",".join(["1"] * n) + ",", "  ISYM=1,", " &END"]
    out = []
    for p in range(n):
        for q in range(p + 1):
            pq = p * (p + 1) // 2 + q
            for r in range(n):
                for s in range(r + 1):
                    rs = r * (r + 1) // 2 + s
                    if rs > pq:
                        continue
                    v = g[p, q, r, s]
                    if abs(v) < 1e-9:
                        continue
                    out.append("%.17e %d %d %d %d" % (v, p + 1, q + 1, r + 1, s + 1))
    for p in range(n):
        for q in range(p + 1):
            v = h[p, q]
            if abs(v) < 1e-9:
                continue
            out.append("%.17e %d %d 0 0" % (v, p + 1, q + 1))
    out.append("%.17e 0 0 0 0" % e_core)
    with open(path, "w") as f:
        f.write("\n".join(lines + out) + "\n")


def make(path, n, n_elec, seed):
    """Writes the synthetic FCIDUMP for (n, seed) to path (skips if it exists)."""
    if os.path.exists(path):
        return path
    h, g = integrals(n, seed)
    tmp = path + ".tmp%d" % os.getpid()
    write_fcidump(tmp, h, g, n_elec)
    os.replace(tmp, path)
    return path


def workload_fcidump(k, directory):
    w = WORKLOADS[k]
    os.makedirs(directory, exist_ok=True)
    path = os.path.join(directory, "FCIDUMP_w%d_n%d" % (k, w["n"]))
    return make(path, w["n"], w["n_up"] + w["n_dn"], BASE_SEED + k)


def batch_instance(i, directory):
    """Small instance i of the batched workload: n ~ U[12, 20], n_up = n_dn ~ U[3, n/2 - 1]."""
    rng = np.random.default_rng(BASE_SEED + 1000 + i)
    n = int(rng.integers(12, 21))
    ne = int(rng.integers(3, n // 2))
    os.makedirs(directory, exist_ok=True)
    path = os.path.join(directory, "FCIDUMP_b%d_n%d" % (i, n))
    make(path, n, 2 * ne, BASE_SEED + 1000 + i)
    return path, n, ne
