"""ctypes binding to libshci_gpu.so (the C ABI declared in include/shci_gpu.h).

There is no CPU fallback: if the library is missing, or no GPU is present, the calls fail
with an exception naming the cause.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libshci_gpu.so")
HEADER = os.path.join(HERE, "..", "include", "shci_gpu.h")

PREC_FP64 = 0
PREC_MIXED = 1

STATUS = {0: "SHCI_OK", 1: "SHCI_ERR_OOM", 2: "SHCI_ERR_ARG", 3: "SHCI_ERR_CUDA",
          4: "SHCI_ERR_TIMEOUT", 5: "SHCI_ERR_OVERFLOW", 6: "SHCI_ERR_CHECK", 7: "SHCI_ERR_IO"}

_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")

_lib = None


class ShciError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


def load():
    """Loads the library (building it first if needed); raises if that is impossible."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _build
        _build.build()
    L = ctypes.CDLL(LIB_PATH)
    vp, sz, d, i, u = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double, ctypes.c_int, ctypes.c_uint
    u64 = ctypes.c_uint64
    P = ctypes.POINTER
    sig = {
        "shci_create": [P(vp), i, sz],
        "shci_destroy": [vp],
        "shci_load_fcidump": [vp, ctypes.c_char_p, u, u, ctypes.c_char_p, i, vp, vp],
        "shci_set_integrals": [vp, i, u, u, d, _f64p, _f64p, vp, ctypes.c_char_p, u64, u64],
        "shci_save_integrals_cache": [vp, ctypes.c_char_p, P(i)],
        "shci_load_integrals_cache": [vp, ctypes.c_char_p, u, u, ctypes.c_char_p, P(i)],
        "shci_get_integrals": [vp, P(i), P(d), vp, vp, vp, vp],
        "shci_get_hf": [vp, P(u64), P(u64), P(d)],
        "shci_build_queues": [vp, _f64p],
        "shci_set_dets": [vp, _u64p, _u64p, vp, sz],
        "shci_get_n_dets": [vp, P(sz)],
        "shci_get_dets": [vp, _u64p, _u64p, vp, sz],
        "shci_set_coefs": [vp, _f64p, sz],
        "shci_set_coefs_dev": [vp, vp, sz],
        "shci_hamiltonian_elems": [vp, _u64p, _u64p, _u64p, _u64p, sz, _f64p],
        "shci_hamiltonian_elems_noalloc": [vp, _u64p, _u64p, _u64p, _u64p, sz, _f64p],
        "shci_update_hamiltonian": [vp, i, P(sz)],
        "shci_get_hamiltonian": [vp, _u64p, _u32p, _f64p, _f64p],
        "shci_get_hamiltonian_rows": [vp, _u64p, sz, _u64p, vp, vp],
        "shci_hv": [vp, vp, vp, i],
        "shci_hv_host": [vp, _f64p, _f64p, i],
        "shci_davidson": [vp, d, P(d), P(i), _f64p, sz, P(sz)],
        "shci_energy_fp64": [vp, P(d)],
        "shci_davidson_csr": [vp, sz, _u64p, _u32p, _f64p, _f64p, _f64p, d, P(d), _f64p, P(i)],
        "shci_select": [vp, d, i, P(sz)],
        "shci_get_eps_tried": [vp, _f64p, sz],
        "shci_set_second_rejection": [vp, i, d],
        "shci_set_has_double_excitation": [vp, i],
        "shci_set_active_space": [vp, vp, sz],
        "shci_get_inactive_orbitals": [vp, P(u64)],
        "shci_set_var_sd": [vp, i],
        "shci_set_hf_options": [vp, i, vp, vp, vp, sz],
        "shci_get_s2": [vp, P(d)],
        "shci_natural_orbitals": [vp, _f64p, _f64p],
        "shci_rotate_integrals": [vp, _f64p],
        "shci_orbital_hessian_diagonal": [vp, _u32p, _u32p, sz, _f64p],
        "shci_orbital_rotation": [vp, _u32p, _u32p, _f64p, sz, _f64p],
        "shci_set_n_states": [vp, u],
        "shci_set_time_sym": [vp, i],
        "shci_unpack_time_sym": [vp],
        "shci_generalized_fock": [vp, _f64p],
        "shci_orbital_parameters": [vp, vp, vp, sz, P(sz)],
        "shci_orbital_gradient": [vp, vp, vp, sz, _f64p],
        "shci_get_state_coefs": [vp, u, _f64p, sz],
        "shci_set_state_coefs": [vp, u, _f64p, sz],
        "shci_get_state_energies": [vp, _f64p, sz],
        "shci_get_var_trace_states": [vp, vp, sz, P(sz)],
        "shci_davidson_csr_states": [vp, sz, _u64p, _u32p, _f64p, _f64p, u, _f64p, d, _f64p,
                                     _f64p, P(i)],
        "shci_run_variation": [vp, _f64p, sz, vp, sz, d, i, _f64p],
        "shci_get_var_trace": [vp, _u64p, _u64p, _f64p, sz, P(sz)],
        "shci_get_launch_count": [vp, P(u64)],
        "shci_pt2_dtm": [vp, d, d, sz, P(d), P(d), P(sz)],
        "shci_hamiltonian_stats": [vp, _u64p],
        "shci_memory_stats": [vp, _u64p],
        "shci_pt2_psto": [vp, d, d, d, sz, d, d, P(d), P(d), P(sz), P(sz)],
        "shci_pt2_psto_auto_batches": [vp, d, d, d, P(sz), P(sz)],
        "shci_pt2_sto": [vp, d, d, d, sz, sz, i, u, sz, d, d, d, d, P(d), P(d), P(sz), _u64p, _f64p, sz],
        "shci_pt_mem_avail": [vp, d, P(d)],
        "shci_mapreduce_sum": [vp, _f64p, sz, _f64p],
        "shci_find_connected_dets": [vp, _u64p, _u64p, _f64p, _f64p, sz, _u64p, vp, vp, vp],
        "shci_rdm1": [vp, _f64p],
        "shci_rdm2": [vp, _f64p],
        "shci_profile": [vp, i],
        "shci_profile_get": [vp, vp, _f64p, _u64p, sz, P(sz)],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.restype = ctypes.c_int
        fn.argtypes = args
    L.shci_last_error.restype = ctypes.c_char_p
    L.shci_last_error.argtypes = [vp]
    L.shci_stream.restype = vp
    L.shci_stream.argtypes = [vp]
    _lib = L
    return L


class BatchItem(ctypes.Structure):
    _fields_ = [("fcidump", ctypes.c_char_p), ("n_up", ctypes.c_uint), ("n_dn", ctypes.c_uint),
                ("point_group", ctypes.c_char_p), ("eps_vars", ctypes.POINTER(ctypes.c_double)),
                ("n_eps", ctypes.c_size_t), ("schedule", ctypes.POINTER(ctypes.c_double)),
                ("n_sched", ctypes.c_size_t), ("target_error", ctypes.c_double),
                ("eps_pt_dtm", ctypes.c_double), ("eps_pt_psto", ctypes.c_double),
                ("eps_pt", ctypes.c_double), ("precision", ctypes.c_int)]


class BatchResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("energy_hf", ctypes.c_double),
                ("energy_var", ctypes.c_double), ("correction_pt", ctypes.c_double),
                ("uncert_pt", ctypes.c_double), ("n_dets", ctypes.c_uint64),
                ("n_pt_dets", ctypes.c_uint64), ("seconds", ctypes.c_double)]


def batch_solve(instances, eps_vars, schedule=(), eps_pt=(0.0, 0.0, 0.0), target_error=5e-5,
                precision=PREC_FP64, n_workers=0, device=0):
    """Solves many small instances concurrently (shci_batch_solve).  instances: list of
    (fcidump_path, n_up, n_dn[, point_group]).  eps_pt = (eps_pt_dtm, eps_pt_psto, eps_pt).
    Returns (list of result dicts, workers used)."""
    L = load()
    L.shci_batch_solve.restype = ctypes.c_int
    L.shci_batch_solve.argtypes = [ctypes.c_int, ctypes.POINTER(BatchItem), ctypes.c_size_t,
                                   ctypes.c_int, ctypes.POINTER(BatchResult),
                                   ctypes.POINTER(ctypes.c_int)]
    n = len(instances)
    ev = (ctypes.c_double * len(eps_vars))(*eps_vars)
    sc = (ctypes.c_double * max(1, len(schedule)))(*schedule)
    items = (BatchItem * n)()
    keep = []
    for k, inst in enumerate(instances):
        path, nu, nd = inst[0], inst[1], inst[2]
        pg = inst[3] if len(inst) > 3 else "C1"
        p, g = str(path).encode(), pg.encode()
        keep += [p, g]
        items[k] = BatchItem(p, nu, nd, g, ev, len(eps_vars), sc, len(schedule), target_error,
                             eps_pt[0], eps_pt[1], eps_pt[2], precision)
    res = (BatchResult * n)()
    used = ctypes.c_int()
    st = L.shci_batch_solve(device, items, n, n_workers, res, ctypes.byref(used))
    out = [dict(status=r.status, energy_hf=r.energy_hf, energy_var=r.energy_var,
                correction_pt=r.correction_pt, uncert_pt=r.uncert_pt, n_dets=r.n_dets,
                n_pt_dets=r.n_pt_dets, seconds=r.seconds) for r in res]
    if st != 0:
        raise ShciError(st, "batch solve failed (per-instance status in the results)")
    return out, used.value


def header_symbols():
    """Names of the functions declared in include/shci_gpu.h."""
    import re
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(shci_[a-z0-9_]+)\s*\(", txt)))


class Context:
    """One SHCI instance on one GPU (owns all device memory of the instance)."""

    def __init__(self, device=0, hbm_budget=0):
        self.L = load()
        h = ctypes.c_void_p()
        st = self.L.shci_create(ctypes.byref(h), device, hbm_budget)
        if st != 0:
            raise ShciError(st, "shci_create failed (is a CUDA GPU visible?)")
        self.h = h
        self._keep = []

    def close(self):
        if getattr(self, "h", None):
            self.L.shci_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _ck(self, st):
        if st != 0:
            raise ShciError(st, self.L.shci_last_error(self.h).decode())

    # ---- integrals -------------------------------------------------------------------
    def load_fcidump(self, path, n_up, n_dn, point_group="C1", reorder=-1, occs_up=None,
                     occs_dn=None):
        ou = od = None
        if occs_up is not None:
            a = np.ascontiguousarray(occs_up, np.uint32)
            b = np.ascontiguousarray(occs_dn, np.uint32)
            self._keep += [a, b]
            ou, od = a.ctypes.data, b.ctypes.data
        self._ck(self.L.shci_load_fcidump(self.h, str(path).encode(), n_up, n_dn,
                                          point_group.encode(), reorder, ou, od))
        self.n_up, self.n_dn = n_up, n_dn
        n = ctypes.c_int()
        self._ck(self.L.shci_get_integrals(self.h, ctypes.byref(n), None, None, None, None, None))
        self.n_orbs = n.value

    def save_integrals_cache(self, path):
        """Writes the integrals cache; False when a file of another format is there."""
        w = ctypes.c_int()
        self._ck(self.L.shci_save_integrals_cache(self.h, str(path).encode(), ctypes.byref(w)))
        return bool(w.value)

    def load_integrals_cache(self, path, n_up, n_dn, point_group="C1"):
        """Loads the integrals cache; False (context unchanged) when missing or foreign."""
        ok = ctypes.c_int()
        self._ck(self.L.shci_load_integrals_cache(self.h, str(path).encode(), n_up, n_dn,
                                                  point_group.encode(), ctypes.byref(ok)))
        if ok.value:
            self.n_up, self.n_dn = n_up, n_dn
            n = ctypes.c_int()
            self._ck(self.L.shci_get_integrals(self.h, ctypes.byref(n), None, None, None, None,
                                               None))
            self.n_orbs = n.value
        return bool(ok.value)

    def set_integrals(self, h1, g2, n_up, n_dn, hf_up, hf_dn, e_core=0.0, orb_sym=None,
                      point_group="C1"):
        n = h1.shape[0]
        sym = None
        if orb_sym is not None:
            s = np.ascontiguousarray(orb_sym, np.uint32)
            self._keep.append(s)
            sym = s.ctypes.data
        self._ck(self.L.shci_set_integrals(self.h, n, n_up, n_dn, e_core,
                                           np.ascontiguousarray(h1, np.float64).ravel(),
                                           np.ascontiguousarray(g2, np.float64).ravel(), sym,
                                           point_group.encode(), hf_up, hf_dn))
        self.n_up, self.n_dn, self.n_orbs = n_up, n_dn, n

    def integrals(self):
        n = self.n_orbs
        h1 = np.zeros((n, n))
        g2 = np.zeros((n, n, n, n))
        sym = np.zeros(n, np.uint32)
        order = np.zeros(n, np.uint32)
        ec = ctypes.c_double()
        self._ck(self.L.shci_get_integrals(self.h, None, ctypes.byref(ec), h1.ctypes.data,
                                           g2.ctypes.data, sym.ctypes.data, order.ctypes.data))
        return h1, g2, sym, order, ec.value

    def hf(self):
        u, d, e = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_double()
        self._ck(self.L.shci_get_hf(self.h, ctypes.byref(u), ctypes.byref(d), ctypes.byref(e)))
        return u.value, d.value, e.value

    def build_queues(self):
        info = np.zeros(4)
        self._ck(self.L.shci_build_queues(self.h, info))
        return dict(max_hci=info[0], n_hci=int(info[1]), max_singles=info[2],
                    n_singles=int(info[3]))

    # ---- dets ------------------------------------------------------------------------
    def set_dets(self, up, dn, coefs=None):
        up = np.ascontiguousarray(up, np.uint64)
        dn = np.ascontiguousarray(dn, np.uint64)
        c = None
        if coefs is not None:
            cc = np.ascontiguousarray(coefs, np.float64)
            self._keep.append(cc)
            c = cc.ctypes.data
        self._ck(self.L.shci_set_dets(self.h, up, dn, c, len(up)))

    def n_dets(self):
        n = ctypes.c_size_t()
        self._ck(self.L.shci_get_n_dets(self.h, ctypes.byref(n)))
        return n.value

    def dets(self):
        n = self.n_dets()
        up = np.zeros(n, np.uint64)
        dn = np.zeros(n, np.uint64)
        c = np.zeros(n)
        self._ck(self.L.shci_get_dets(self.h, up, dn, c.ctypes.data, n))
        return up, dn, c

    def set_coefs(self, c):
        c = np.ascontiguousarray(c, np.float64)
        self._ck(self.L.shci_set_coefs(self.h, c, len(c)))

    def set_coefs_dev(self, ptr, n):
        self._ck(self.L.shci_set_coefs_dev(self.h, ptr, n))

    def h_elems(self, ui, di, uj, dj):
        ui, di, uj, dj = (np.ascontiguousarray(x, np.uint64) for x in (ui, di, uj, dj))
        out = np.zeros(len(ui))
        self._ck(self.L.shci_hamiltonian_elems(self.h, ui, di, uj, dj, len(ui), out))
        return out

    def h_elems_noalloc(self, ui, di, uj, dj):
        """shci_hamiltonian_elems_noalloc: same results, staged in the library's fixed device
        array (no device allocation; at most 65,536 pairs per call)."""
        ui, di, uj, dj = (np.ascontiguousarray(x, np.uint64) for x in (ui, di, uj, dj))
        out = np.zeros(len(ui))
        self._ck(self.L.shci_hamiltonian_elems_noalloc(self.h, ui, di, uj, dj, len(ui), out))
        return out

    # ---- Hamiltonian / Davidson --------------------------------------------------------
    def update_hamiltonian(self, precision=PREC_FP64):
        nnz = (ctypes.c_size_t * 2)()
        self._ck(self.L.shci_update_hamiltonian(self.h, precision, nnz))
        return nnz[0], nnz[1]

    def hamiltonian_stats(self):
        s = np.zeros(10, np.uint64)
        self._ck(self.L.shci_hamiltonian_stats(self.h, s))
        if int(s[9]) == 1:
            return dict(path="core_join", n=int(s[0]), nnz=int(s[1]), candidates=int(s[5]),
                        core_entries=int(s[6]), one_pass=bool(s[7]))
        return dict(path="group_scan", n=int(s[0]), nnz=int(s[1]), n_alpha=int(s[2]),
                    n_beta=int(s[3]), alpha_singles=int(s[4]), candidates=int(s[5]),
                    cand_same_beta=int(s[6]), cand_same_alpha=int(s[7]), cand_mixed=int(s[8]))

    def memory_stats(self):
        """(bytes held now, peak bytes held, budget) of the context's device memory (the bytes
        held include the context's cache of released blocks: memory_cached())."""
        m = np.zeros(5, np.uint64)
        self._ck(self.L.shci_memory_stats(self.h, m))
        return int(m[0]), int(m[1]), int(m[2])

    def memory_cached(self):
        """(bytes in the cache of released blocks, peak bytes held by live buffers)"""
        m = np.zeros(5, np.uint64)
        self._ck(self.L.shci_memory_stats(self.h, m))
        return int(m[3]), int(m[4])

    def hamiltonian_rows(self, rows):
        """Elements of the given rows (strict upper part): offsets, cols, FP64 values, each row
        in increasing column order."""
        rows = np.ascontiguousarray(rows, np.uint64)
        off = np.zeros(len(rows) + 1, np.uint64)
        self._ck(self.L.shci_get_hamiltonian_rows(self.h, rows, len(rows), off, None, None))
        m = int(off[-1])
        cols = np.zeros(max(m, 1), np.uint32)
        vals = np.zeros(max(m, 1))
        self._ck(self.L.shci_get_hamiltonian_rows(self.h, rows, len(rows), off, cols.ctypes.data,
                                                  vals.ctypes.data))
        return off, cols[:m], vals[:m]

    def hamiltonian(self, nnz):
        n = self.n_dets()
        rp = np.zeros(n + 1, np.uint64)
        cols = np.zeros(max(nnz, 1), np.uint32)
        vals = np.zeros(max(nnz, 1))
        diag = np.zeros(n)
        self._ck(self.L.shci_get_hamiltonian(self.h, rp, cols, vals, diag))
        return rp, cols[:nnz], vals[:nnz], diag

    def hv(self, x, residual=False):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self._ck(self.L.shci_hv_host(self.h, x, y, int(residual)))
        return y

    def hv_dev(self, x_ptr, y_ptr, residual=False):
        self._ck(self.L.shci_hv(self.h, x_ptr, y_ptr, int(residual)))

    def davidson(self, tol):
        e = ctypes.c_double()
        conv = ctypes.c_int()
        tr = np.zeros(64)
        nt = ctypes.c_size_t()
        self._ck(self.L.shci_davidson(self.h, tol, ctypes.byref(e), ctypes.byref(conv), tr, 64,
                                      ctypes.byref(nt)))
        return e.value, bool(conv.value), tr[: nt.value]

    def energy_fp64(self):
        e = ctypes.c_double()
        self._ck(self.L.shci_energy_fp64(self.h, ctypes.byref(e)))
        return e.value

    def davidson_csr(self, row_ptr, cols, vals, diag, init, tol):
        n = len(diag)
        e = ctypes.c_double()
        conv = ctypes.c_int()
        vec = np.zeros(n)
        self._ck(self.L.shci_davidson_csr(self.h, n, np.ascontiguousarray(row_ptr, np.uint64),
                                          np.ascontiguousarray(cols, np.uint32),
                                          np.ascontiguousarray(vals, np.float64),
                                          np.ascontiguousarray(diag, np.float64),
                                          np.ascontiguousarray(init, np.float64), tol,
                                          ctypes.byref(e), vec, ctypes.byref(conv)))
        return e.value, vec, bool(conv.value)

    # ---- selection / variation / PT2 ------------------------------------------------------
    def select(self, eps_var, var_sd=False):
        n = ctypes.c_size_t()
        self._ck(self.L.shci_select(self.h, eps_var, int(var_sd), ctypes.byref(n)))
        return n.value

    def generalized_fock(self):
        n = self.n_orbs
        F = np.zeros(n * n)
        self._ck(self.L.shci_generalized_fock(self.h, F))
        return F.reshape(n, n)

    def orbital_parameters(self):
        k = ctypes.c_size_t()
        self._ck(self.L.shci_orbital_parameters(self.h, None, None, 0, ctypes.byref(k)))
        p = np.zeros(k.value, np.uint32)
        q = np.zeros(k.value, np.uint32)
        self._ck(self.L.shci_orbital_parameters(self.h, p.ctypes.data, q.ctypes.data, k.value,
                                                ctypes.byref(k)))
        return p, q

    def orbital_gradient(self, p, q):
        p = np.ascontiguousarray(p, np.uint32)
        q = np.ascontiguousarray(q, np.uint32)
        g = np.zeros(len(p))
        self._ck(self.L.shci_orbital_gradient(self.h, p.ctypes.data, q.ctypes.data, len(p), g))
        return g

    def set_time_sym(self, on=True):
        self._ck(self.L.shci_set_time_sym(self.h, int(on)))

    def unpack_time_sym(self):
        self._ck(self.L.shci_unpack_time_sym(self.h))

    def set_n_states(self, n):
        self._ck(self.L.shci_set_n_states(self.h, n))
        self.n_states = n

    def state_coefs(self, s):
        n = self.n_dets()
        out = np.zeros(n)
        self._ck(self.L.shci_get_state_coefs(self.h, s, out, n))
        return out

    def set_state_coefs(self, s, c):
        c = np.ascontiguousarray(c, np.float64)
        self._ck(self.L.shci_set_state_coefs(self.h, s, c, len(c)))

    def state_energies(self):
        ns = getattr(self, "n_states", 1)
        out = np.zeros(ns)
        self._ck(self.L.shci_get_state_energies(self.h, out, ns))
        return out

    def var_trace_states(self):
        ns = getattr(self, "n_states", 1)
        n = ctypes.c_size_t()
        self._ck(self.L.shci_get_var_trace_states(self.h, None, 0, ctypes.byref(n)))
        out = np.zeros((max(n.value, 1), ns))
        self._ck(self.L.shci_get_var_trace_states(self.h, out.ctypes.data, out.size,
                                                  ctypes.byref(n)))
        return out[: n.value]

    def davidson_csr_states(self, row_ptr, cols, vals, diag, init, tol):
        init = np.ascontiguousarray(init, np.float64)
        ns, n = init.shape
        ev = np.zeros(ns)
        vecs = np.zeros((ns, n))
        conv = ctypes.c_int()
        self._ck(self.L.shci_davidson_csr_states(
            self.h, n, np.ascontiguousarray(row_ptr, np.uint64),
            np.ascontiguousarray(cols, np.uint32), np.ascontiguousarray(vals, np.float64),
            np.ascontiguousarray(diag, np.float64), ns, init, tol, ev, vecs, ctypes.byref(conv)))
        return ev, vecs, bool(conv.value)

    def set_second_rejection(self, enable=True, factor=0.2):
        self._ck(self.L.shci_set_second_rejection(self.h, int(enable), factor))

    def set_has_double_excitation(self, on=True):
        self._ck(self.L.shci_set_has_double_excitation(self.h, int(on)))

    def set_active_space(self, irrep_active_space):
        a = np.ascontiguousarray(irrep_active_space, np.uint32)
        self._ck(self.L.shci_set_active_space(self.h, a.ctypes.data if len(a) else None, len(a)))

    def inactive_orbitals(self):
        m = ctypes.c_uint64()
        self._ck(self.L.shci_get_inactive_orbitals(self.h, ctypes.byref(m)))
        return m.value

    def set_var_sd(self, on=True):
        self._ck(self.L.shci_set_var_sd(self.h, int(on)))

    def set_hf_options(self, allow_doubly_occupy=True, irreps=(), irrep_occs_up=(),
                       irrep_occs_dn=()):
        """HF det options of the next load_fcidump (chem/irreps, allow_doubly_occupy_hf)."""
        a = np.ascontiguousarray(irreps, np.uint32)
        b = np.ascontiguousarray(irrep_occs_up, np.uint32)
        c = np.ascontiguousarray(irrep_occs_dn, np.uint32)
        n = len(a)
        self._ck(self.L.shci_set_hf_options(self.h, int(allow_doubly_occupy),
                                            a.ctypes.data if n else None,
                                            b.ctypes.data if n else None,
                                            c.ctypes.data if n else None, n))

    def natural_orbitals(self):
        """(rotation U with U[i, p], occupation numbers) of the 1-RDM, per irrep."""
        n = self.n_orbs
        rot, occ = np.zeros(n * n), np.zeros(n)
        self._ck(self.L.shci_natural_orbitals(self.h, rot, occ))
        return rot.reshape(n, n), occ

    def orbital_hessian_diagonal(self, p, q):
        p = np.ascontiguousarray(p, np.uint32)
        q = np.ascontiguousarray(q, np.uint32)
        out = np.zeros(len(p))
        self._ck(self.L.shci_orbital_hessian_diagonal(self.h, p, q, len(p), out))
        return out

    def orbital_rotation(self, p, q, kappa):
        n = self.n_orbs
        rot = np.zeros(n * n)
        self._ck(self.L.shci_orbital_rotation(self.h, np.ascontiguousarray(p, np.uint32),
                                              np.ascontiguousarray(q, np.uint32),
                                              np.ascontiguousarray(kappa, np.float64), len(p),
                                              rot))
        return rot.reshape(n, n)

    def rotate_integrals(self, rot):
        self._ck(self.L.shci_rotate_integrals(self.h, np.ascontiguousarray(rot, np.float64).ravel()))

    def s2(self):
        v = ctypes.c_double()
        self._ck(self.L.shci_get_s2(self.h, ctypes.byref(v)))
        return v.value

    def eps_tried(self):
        n = self.n_dets()
        out = np.zeros(n)
        self._ck(self.L.shci_get_eps_tried(self.h, out, n))
        return out

    def run_variation(self, eps_vars, schedule=(), target_error=5e-5, precision=PREC_FP64):
        ev = np.ascontiguousarray(eps_vars, np.float64)
        sc = np.ascontiguousarray(schedule, np.float64)
        out = np.zeros(len(ev))
        self._ck(self.L.shci_run_variation(self.h, ev, len(ev), sc.ctypes.data if len(sc) else None,
                                           len(sc), target_error, precision, out))
        return out

    def var_trace(self):
        n = ctypes.c_size_t()
        self._ck(self.L.shci_get_var_trace(self.h, np.zeros(1, np.uint64), np.zeros(1, np.uint64),
                                           np.zeros(1), 0, ctypes.byref(n)))
        nd = np.zeros(n.value, np.uint64)
        nz = np.zeros(n.value, np.uint64)
        e = np.zeros(n.value)
        self._ck(self.L.shci_get_var_trace(self.h, nd, nz, e, n.value, ctypes.byref(n)))
        return nd, nz, e

    def launches(self):
        n = ctypes.c_uint64()
        self._ck(self.L.shci_get_launch_count(self.h, ctypes.byref(n)))
        return n.value

    def pt2_dtm(self, energy_var, eps_pt_dtm, n_batches=1):
        v, u, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_size_t()
        self._ck(self.L.shci_pt2_dtm(self.h, energy_var, eps_pt_dtm, n_batches, ctypes.byref(v),
                                     ctypes.byref(u), ctypes.byref(n)))
        return v.value, u.value, n.value

    def pt2_psto(self, energy_var, eps_pt_dtm, eps_pt_psto, n_batches=16, target_error=5e-5,
                 eps_pt=0.0):
        v, u, n, b = ctypes.c_double(), ctypes.c_double(), ctypes.c_size_t(), ctypes.c_size_t()
        self._ck(self.L.shci_pt2_psto(self.h, energy_var, eps_pt_dtm, eps_pt_psto, n_batches,
                                      target_error, eps_pt, ctypes.byref(v), ctypes.byref(u),
                                      ctypes.byref(n), ctypes.byref(b)))
        return v.value, u.value, n.value, b.value

    def psto_auto_batches(self, eps_pt_psto, pt_mem_avail, mem_usage=1.0):
        """(batch count, pilot PT dets) of the automatic psto batch count."""
        nb, npd = ctypes.c_size_t(), ctypes.c_size_t()
        self._ck(self.L.shci_pt2_psto_auto_batches(self.h, eps_pt_psto, pt_mem_avail, mem_usage,
                                                   ctypes.byref(nb), ctypes.byref(npd)))
        return nb.value, npd.value

    def pt2_sto(self, energy_var, eps_pt_psto, eps_pt, n_batches, n_samples, seed=347634253,
                max_iter=100, target_error=5e-5, psto_uncert=0.0, semisto=False,
                pt_mem_avail=0.0, mem_usage=0.4, info=None):
        """n_samples = 0: the reference's pilot sizes the sample from pt_mem_avail (bytes);
        info (a dict, optional) receives n_samples, n_dtm and n_unique_target."""
        v, u, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_size_t()
        loops = np.zeros(max_iter)
        si = np.zeros(3, np.uint64)
        self._ck(self.L.shci_pt2_sto(self.h, energy_var, eps_pt_psto, eps_pt, n_batches,
                                     n_samples, int(semisto), seed, max_iter, target_error,
                                     psto_uncert, float(pt_mem_avail), mem_usage,
                                     ctypes.byref(v), ctypes.byref(u), ctypes.byref(n), si,
                                     loops, max_iter))
        if info is not None:
            info.update(n_samples=int(si[0]), n_dtm=int(si[1]), n_unique_target=int(si[2]))
        return v.value, u.value, loops[: n.value]

    def pt_mem_avail(self, mem_total):
        out = ctypes.c_double()
        self._ck(self.L.shci_pt_mem_avail(self.h, float(mem_total), ctypes.byref(out)))
        return out.value

    def find_connected(self, up, dn, eps_max, eps_min):
        """BaseSystem::find_connected_dets for each det: (offsets[n+1], up, dn, n_excite)."""
        up = np.ascontiguousarray(up, np.uint64)
        dn = np.ascontiguousarray(dn, np.uint64)
        n = len(up)
        hi = np.ascontiguousarray(np.broadcast_to(eps_max, (n,)), np.float64)
        lo = np.ascontiguousarray(np.broadcast_to(eps_min, (n,)), np.float64)
        off = np.zeros(n + 1, np.uint64)
        self._ck(self.L.shci_find_connected_dets(self.h, up, dn, hi, lo, n, off, None, None,
                                                 None))
        m = int(off[-1])
        cu = np.zeros(max(m, 1), np.uint64)
        cd = np.zeros(max(m, 1), np.uint64)
        nx = np.zeros(max(m, 1), np.uint8)
        self._ck(self.L.shci_find_connected_dets(self.h, up, dn, hi, lo, n, off,
                                                 cu.ctypes.data, cd.ctypes.data,
                                                 nx.ctypes.data))
        return off, cu[:m], cd[:m], nx[:m]

    def mapreduce_sum(self, x):
        """(sum x, sum x^2) by the PT2 stages' compensated device reduction."""
        x = np.ascontiguousarray(x, np.float64)
        out = np.zeros(2)
        self._ck(self.L.shci_mapreduce_sum(self.h, x, len(x), out))
        return out[0], out[1]

    def rdm1(self):
        n = self.n_orbs
        out = np.zeros(n * n)
        self._ck(self.L.shci_rdm1(self.h, out))
        return out.reshape(n, n)

    def rdm2_half(self):
        n = self.n_orbs
        out = np.zeros(n * n * (n * n + 1) // 2)
        self._ck(self.L.shci_rdm2(self.h, out))
        return out

    def stream(self):
        return self.L.shci_stream(self.h)

    def profile(self, enable=True):
        self._ck(self.L.shci_profile(self.h, int(enable)))

    def profile_get(self):
        """{stage: (total_ms, launches)} recorded since profiling was enabled."""
        cap = 64
        names = ctypes.create_string_buffer(32 * cap)
        ms = np.zeros(cap)
        cnt = np.zeros(cap, np.uint64)
        n = ctypes.c_size_t()
        self._ck(self.L.shci_profile_get(self.h, ctypes.cast(names, ctypes.c_void_p), ms, cnt,
                                         cap, ctypes.byref(n)))
        out = {}
        for k in range(min(n.value, cap)):
            nm = names.raw[32 * k:32 * k + 32].split(b"\0")[0].decode()
            out[nm] = (float(ms[k]), int(cnt[k]))
        return out
