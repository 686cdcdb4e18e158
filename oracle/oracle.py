"""ctypes wrapper around the SHCI oracle (oracle/shci_oracle.cc).

TEST INFRASTRUCTURE ONLY.  The oracle is a CPU restatement of the reference's algorithm
(QMC-Cornell/shci); only tests/, the smoke check and the bench's CPU-baseline leg use it, and
only as the checker.  The product library never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liboracle.so")
_REF = os.path.join(_HERE, "_ref", "libref_pin.so")

_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def reference_dir():
    """The reference checkout: $SHCI_REFERENCE, else /root/reference (may be absent)."""
    return os.environ.get("SHCI_REFERENCE", "/root/reference")


def build(ref=True):
    """Compile the oracle (and, when the reference tree is present, the reference pin)."""
    subprocess.run(["make", "-s", "-C", _HERE, "all"], check=True)
    r = reference_dir()
    if ref and os.path.isdir(os.path.join(r, "src")):
        subprocess.run(["make", "-s", "-C", _HERE, "ref", "REF=" + r], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build(ref=False)
        L = ctypes.CDLL(_LIB)
        vp, sz, d, u, i = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double, ctypes.c_uint, ctypes.c_int
        u64 = ctypes.c_uint64
        sig = {
            "orc_create": (vp, [ctypes.c_char_p, u, u, ctypes.c_char_p, i, vp, vp, ctypes.c_char_p, sz]),
            "orc_destroy": (None, [vp]),
            "orc_set_threads": (None, [i]),
            "orc_n_orbs": (u, [vp]),
            "orc_info": (None, [vp, _f64p]),
            "orc_hf": (None, [vp, ctypes.POINTER(u64), ctypes.POINTER(u64)]),
            "orc_integrals": (None, [vp, vp, vp, vp, vp]),
            "orc_hamiltonian_elem": (d, [vp, u64, u64, u64, u64, i]),
            "orc_diff": (None, [u64, u64, _u32p, ctypes.POINTER(ctypes.c_int)]),
            "orc_det_hash": (u64, [u64, u64]),
            "orc_rehash": (u64, [u64]),
            "orc_find_connected": (sz, [vp, u64, u64, d, d, _u64p, _u64p, _i32p, sz]),
            "orc_hci_queue": (sz, [vp, sz, _f64p, _u32p, _u32p, sz]),
            "orc_singles_queue": (sz, [vp, u, _f64p, _u32p, sz]),
            "orc_set_dets": (None, [vp, _u64p, _u64p, vp, sz]),
            "orc_n_dets": (sz, [vp]),
            "orc_get_dets": (None, [vp, _u64p, _u64p, vp]),
            "orc_set_coefs": (None, [vp, _f64p]),
            "orc_update_hamiltonian": (sz, [vp]),
            "orc_clear_hamiltonian": (None, [vp]),
            "orc_get_hamiltonian": (None, [vp, _u64p, _u32p, _f64p]),
            "orc_hv": (None, [vp, _f64p, _f64p]),
            "orc_davidson": (i, [vp, _f64p, d, ctypes.POINTER(d), _f64p, sz, ctypes.POINTER(sz)]),
            "orc_davidson_csr": (i, [sz, _u64p, _u32p, _f64p, _f64p, d, ctypes.POINTER(d)]),
            "orc_davidson_csr_states": (i, [sz, _u64p, _u32p, _f64p, u, _f64p, d, _f64p, _f64p]),
            "orc_set_n_states": (None, [vp, u]),
            "orc_set_time_sym": (None, [vp, i]),
            "orc_set_second_rejection": (None, [vp, i]),
            "orc_create_hf": (vp, [ctypes.c_char_p, u, u, ctypes.c_char_p, i, i, vp, vp, vp, u,
                                   ctypes.c_char_p, sz]),
            "orc_set_has_double_excitation": (None, [vp, i]),
            "orc_set_active_space": (None, [vp, vp, u]),
            "orc_get_s2": (d, [vp]),
            "orc_set_var_sd": (None, [vp, i]),
            "orc_unpack_time_sym": (None, [vp]),
            "orc_generalized_fock": (None, [vp, _f64p, _f64p, _f64p]),
            "orc_orbital_parameters": (sz, [vp, vp, vp, sz]),
            "orc_get_state_coefs": (None, [vp, u, _f64p]),
            "orc_set_state_coefs": (None, [vp, u, _f64p]),
            "orc_state_energies": (None, [vp, _f64p, vp]),
            "orc_select": (sz, [vp, d, i]),
            "orc_eps_tried": (None, [vp, _f64p]),
            "orc_run_all_variations": (None, [vp, _f64p, sz, _f64p, sz, d, i, _f64p]),
            "orc_n_iterations": (sz, [vp]),
            "orc_iterations": (None, [vp, _u64p, _u64p, _f64p]),
            "orc_energy_var": (d, [vp]),
            "orc_set_energy_var": (None, [vp, d]),
            "orc_pt_dtm": (None, [vp, d, sz, ctypes.POINTER(d), ctypes.POINTER(d), ctypes.POINTER(sz)]),
            "orc_run_variation_step": (d, [vp, d, i, d]),
            "orc_hbuild_sample": (None, [vp, sz, sz, _f64p]),
            "orc_sample_rows": (sz, [vp, vp, vp, vp, vp]),
            "orc_threads": (i, []),
            "orc_pt_psto": (None, [vp, d, d, sz, d, d, _f64p]),
            "orc_pt_sto": (sz, [vp, d, d, sz, sz, u, sz, d, d, i, d, d, _f64p, _f64p, sz]),
            "orc_rdm1": (None, [vp, _f64p]),
            "orc_rdm2": (None, [vp, _f64p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def ref_pin():
    """The reference's own det/hash/alias routines (None when not built here)."""
    if not os.path.exists(_REF):
        return None
    L = ctypes.CDLL(_REF)
    u64 = ctypes.c_uint64
    L.ref_half_hash.restype = u64
    L.ref_half_hash.argtypes = [u64]
    L.ref_det_hash.restype = u64
    L.ref_det_hash.argtypes = [u64, u64]
    L.ref_rehash.restype = u64
    L.ref_rehash.argtypes = [u64]
    L.ref_diff.restype = None
    L.ref_diff.argtypes = [u64, u64, _u32p, ctypes.POINTER(ctypes.c_int)]
    L.ref_n_diffs.restype = ctypes.c_uint
    L.ref_n_diffs.argtypes = [u64, u64]
    L.ref_bit_till.restype = ctypes.c_uint
    L.ref_bit_till.argtypes = [u64, ctypes.c_uint]
    L.ref_det_less.restype = ctypes.c_int
    L.ref_det_less.argtypes = [u64, u64, u64, u64]
    L.ref_alias.restype = None
    L.ref_alias.argtypes = [_f64p, ctypes.c_size_t, _f64p, _u64p]
    return L


class Oracle:
    """One SHCI system (integrals, queues, dets, Hamiltonian) in the CPU restatement."""

    def __init__(self, fcidump, n_up, n_dn, point_group="C1", reorder=-1, occs_up=None,
                 occs_dn=None, allow_doubly_occupy=True, irreps=None, irrep_occs_up=None,
                 irrep_occs_dn=None):
        L = lib()
        err = ctypes.create_string_buffer(512)
        self._keep = []
        ou = od = None
        if occs_up is not None:
            a = np.ascontiguousarray(occs_up, dtype=np.uint32)
            b = np.ascontiguousarray(occs_dn, dtype=np.uint32)
            self._keep += [a, b]
            ou, od = a.ctypes.data, b.ctypes.data
        if occs_up is None and (irreps is not None or not allow_doubly_occupy):
            ir = np.ascontiguousarray(irreps if irreps is not None else [], dtype=np.uint32)
            iu = np.ascontiguousarray(irrep_occs_up if irreps is not None else [], np.uint32)
            idn = np.ascontiguousarray(irrep_occs_dn if irreps is not None else [], np.uint32)
            self._keep += [ir, iu, idn]
            self.h = L.orc_create_hf(str(fcidump).encode(), n_up, n_dn, point_group.encode(),
                                     reorder, int(allow_doubly_occupy), ir.ctypes.data,
                                     iu.ctypes.data, idn.ctypes.data, len(ir), err, 512)
        else:
            self.h = L.orc_create(str(fcidump).encode(), n_up, n_dn, point_group.encode(),
                                  reorder, ou, od, err, 512)
        if not self.h:
            raise RuntimeError("oracle: " + err.value.decode())
        self.L = L
        self.n_orbs = L.orc_n_orbs(self.h)
        self.n_up, self.n_dn = n_up, n_dn

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    @staticmethod
    def set_threads(n):
        lib().orc_set_threads(n)

    def info(self):
        out = np.zeros(6)
        self.L.orc_info(self.h, out)
        return dict(energy_hf=out[0], max_hci=out[1], n_hci=int(out[2]), max_singles=out[3],
                    n_singles=int(out[4]), energy_core=out[5])

    def hf(self):
        u, d = ctypes.c_uint64(), ctypes.c_uint64()
        self.L.orc_hf(self.h, ctypes.byref(u), ctypes.byref(d))
        return u.value, d.value

    def integrals(self):
        n = self.n_orbs
        h1 = np.zeros((n, n))
        g2 = np.zeros((n, n, n, n))
        sym = np.zeros(n, dtype=np.uint32)
        order = np.zeros(n, dtype=np.uint32)
        self.L.orc_integrals(self.h, h1.ctypes.data, g2.ctypes.data, sym.ctypes.data,
                             order.ctypes.data)
        return h1, g2, sym, order

    def h_elem(self, di, dj, n_excite=-1):
        return self.L.orc_hamiltonian_elem(self.h, di[0], di[1], dj[0], dj[1], n_excite)

    def find_connected(self, det, eps_max, eps_min, cap=1 << 20):
        up = np.zeros(cap, np.uint64)
        dn = np.zeros(cap, np.uint64)
        nx = np.zeros(cap, np.int32)
        c = self.L.orc_find_connected(self.h, det[0], det[1], eps_max, eps_min, up, dn, nx, cap)
        assert c <= cap
        return up[:c], dn[:c], nx[:c]

    def set_dets(self, up, dn, coefs=None):
        up = np.ascontiguousarray(up, np.uint64)
        dn = np.ascontiguousarray(dn, np.uint64)
        c = None
        if coefs is not None:
            cc = np.ascontiguousarray(coefs, np.float64)
            self._keep.append(cc)
            c = cc.ctypes.data
        self.L.orc_set_dets(self.h, up, dn, c, len(up))

    def dets(self):
        n = self.L.orc_n_dets(self.h)
        up = np.zeros(n, np.uint64)
        dn = np.zeros(n, np.uint64)
        c = np.zeros(n)
        self.L.orc_get_dets(self.h, up, dn, c.ctypes.data)
        return up, dn, c

    def set_coefs(self, c):
        self.L.orc_set_coefs(self.h, np.ascontiguousarray(c, np.float64))

    def generalized_fock(self, g1, half):
        """Optimization::get_generalized_Fock from the given RDMs (n x n)."""
        n = self.n_orbs
        F = np.zeros(n * n)
        self.L.orc_generalized_fock(self.h, np.ascontiguousarray(g1, np.float64).ravel(),
                                    np.ascontiguousarray(half, np.float64), F)
        return F.reshape(n, n)

    def orbital_parameters(self):
        k = self.L.orc_orbital_parameters(self.h, None, None, 0)
        p = np.zeros(k, np.uint32)
        q = np.zeros(k, np.uint32)
        self.L.orc_orbital_parameters(self.h, p.ctypes.data, q.ctypes.data, k)
        return p, q

    def set_time_sym(self, on=True):
        self.L.orc_set_time_sym(self.h, int(on))

    def unpack_time_sym(self):
        self.L.orc_unpack_time_sym(self.h)

    def set_n_states(self, n):
        self.n_states = n
        self.L.orc_set_n_states(self.h, n)

    def state_coefs(self, s):
        out = np.zeros(self.L.orc_n_dets(self.h))
        self.L.orc_get_state_coefs(self.h, s, out)
        return out

    def set_state_coefs(self, s, c):
        self.L.orc_set_state_coefs(self.h, s, np.ascontiguousarray(c, np.float64))

    def state_energies(self):
        """(energies of the states after the last run, per-iteration energies (n_iter, n_states))"""
        ns = getattr(self, "n_states", 1)
        e = np.zeros(ns)
        n_it = self.L.orc_n_iterations(self.h)
        per = np.zeros((max(n_it, 1), ns))
        self.L.orc_state_energies(self.h, e, per.ctypes.data)
        return e, per[:n_it]

    def update_hamiltonian(self):
        return self.L.orc_update_hamiltonian(self.h)

    def clear_hamiltonian(self):
        self.L.orc_clear_hamiltonian(self.h)

    def hamiltonian(self, nnz):
        n = self.L.orc_n_dets(self.h)
        rp = np.zeros(n + 1, np.uint64)
        cols = np.zeros(nnz, np.uint32)
        vals = np.zeros(nnz)
        self.L.orc_get_hamiltonian(self.h, rp, cols, vals)
        return rp, cols, vals

    def hv(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self.L.orc_hv(self.h, x, y)
        return y

    def davidson(self, coefs, tol):
        c = np.array(coefs, np.float64)
        e = ctypes.c_double()
        tr = np.zeros(64)
        nt = ctypes.c_size_t()
        conv = self.L.orc_davidson(self.h, c, tol, ctypes.byref(e), tr, 64, ctypes.byref(nt))
        return e.value, c, bool(conv), tr[: nt.value]

    def set_has_double_excitation(self, on=True):
        self.L.orc_set_has_double_excitation(self.h, int(on))

    def set_active_space(self, irrep_active_space):
        a = np.ascontiguousarray(irrep_active_space, dtype=np.uint32)
        self._keep.append(a)
        self.L.orc_set_active_space(self.h, a.ctypes.data if len(a) else None, len(a))

    def s2(self):
        return self.L.orc_get_s2(self.h)

    def set_var_sd(self, on=True):
        self.L.orc_set_var_sd(self.h, int(on))

    def select(self, eps_var, var_sd=False):
        return self.L.orc_select(self.h, eps_var, int(var_sd))

    def eps_tried(self):
        out = np.zeros(self.L.orc_n_dets(self.h))
        self.L.orc_eps_tried(self.h, out)
        return out

    def run_all_variations(self, eps_vars, schedule=(), target_error=5e-5, second_rejection=False):
        ev = np.ascontiguousarray(eps_vars, np.float64)
        sc = np.ascontiguousarray(schedule if len(schedule) else [0.0], np.float64)
        out = np.zeros(len(ev))
        self.L.orc_run_all_variations(self.h, ev, len(ev), sc, len(schedule), target_error,
                                      int(second_rejection), out)
        return out

    def run_variation_step(self, eps_var, until_converged, target_error=5e-5):
        return self.L.orc_run_variation_step(self.h, eps_var, int(until_converged), target_error)

    def hbuild_sample(self, stride, offset=0):
        out = np.zeros(5)
        self.L.orc_hbuild_sample(self.h, stride, offset, out)
        return dict(index_s=out[0], rows_s=out[1], spmv_s=out[2], nnz=int(out[3]),
                    rows=int(out[4]))

    def sample_rows(self):
        """Rows of the last hbuild_sample: (row ids, offsets, cols, FP64 values), each row's
        strict upper part in increasing column order."""
        m = self.L.orc_sample_rows(self.h, None, None, None, None)
        rows = np.zeros(m, np.uint64)
        off = np.zeros(m + 1, np.uint64)
        self.L.orc_sample_rows(self.h, rows.ctypes.data, off.ctypes.data, None, None)
        t = int(off[-1])
        cols = np.zeros(max(t, 1), np.uint32)
        vals = np.zeros(max(t, 1))
        self.L.orc_sample_rows(self.h, rows.ctypes.data, off.ctypes.data, cols.ctypes.data,
                               vals.ctypes.data)
        return rows, off, cols[:t], vals[:t]

    @staticmethod
    def threads():
        return lib().orc_threads()

    def iterations(self):
        n = self.L.orc_n_iterations(self.h)
        nd = np.zeros(n, np.uint64)
        nz = np.zeros(n, np.uint64)
        e = np.zeros(n)
        self.L.orc_iterations(self.h, nd, nz, e)
        return nd, nz, e

    @property
    def energy_var(self):
        return self.L.orc_energy_var(self.h)

    @energy_var.setter
    def energy_var(self, e):
        self.L.orc_set_energy_var(self.h, e)

    def pt_dtm(self, eps_pt_dtm, n_batches=1):
        v, u, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_size_t()
        self.L.orc_pt_dtm(self.h, eps_pt_dtm, n_batches, ctypes.byref(v), ctypes.byref(u),
                          ctypes.byref(n))
        return v.value, u.value, n.value

    def pt_psto(self, eps_dtm, eps_psto, n_batches, target_error=5e-5, eps_pt=0.0):
        out = np.zeros(4)
        self.L.orc_pt_psto(self.h, eps_dtm, eps_psto, n_batches, target_error, eps_pt, out)
        return out[0], out[1], int(out[2]), int(out[3])

    def pt_sto(self, eps_psto, eps_pt, n_batches, n_samples, seed=347634253, max_iter=100,
               target_error=5e-5, psto_uncert=0.0, semisto=False, pt_mem_avail=0.0,
               mem_usage=0.4, info=None):
        """n_samples = 0: sample size from the reference's pilot and pt_mem_avail (bytes);
        semisto: deterministic top quarter.  info (a dict, optional) receives n_samples,
        n_dtm and n_unique_target."""
        out = np.zeros(5)
        loops = np.zeros(max_iter)
        n = self.L.orc_pt_sto(self.h, eps_psto, eps_pt, n_batches, n_samples, seed, max_iter,
                              target_error, psto_uncert, int(semisto), float(pt_mem_avail),
                              mem_usage, out, loops, max_iter)
        if n == (1 << 64) - 1:
            raise RuntimeError("oracle: semistochastic PT2 needs a sample-size target >= 4")
        if info is not None:
            info.update(n_samples=int(out[2]), n_dtm=int(out[3]), n_unique_target=int(out[4]))
        return out[0], out[1], loops[:n]

    def rdm1(self):
        out = np.zeros(self.n_orbs * self.n_orbs)
        self.L.orc_rdm1(self.h, out)
        return out.reshape(self.n_orbs, self.n_orbs)

    def rdm2_half(self):
        n = self.n_orbs
        out = np.zeros(n * n * (n * n + 1) // 2)
        self.L.orc_rdm2(self.h, out)
        return out


def davidson_csr_states(row_ptr, cols, vals, init, tol):
    """Several-state Davidson (davidson.cc) on an upper-triangle CSR; init is (n_states, n)."""
    init = np.ascontiguousarray(init, np.float64)
    ns, n = init.shape
    ev = np.zeros(ns)
    vecs = np.zeros((ns, n))
    conv = lib().orc_davidson_csr_states(n, np.ascontiguousarray(row_ptr, np.uint64),
                                         np.ascontiguousarray(cols, np.uint32),
                                         np.ascontiguousarray(vals, np.float64), ns, init, tol,
                                         ev, vecs)
    return ev, vecs, bool(conv)


def davidson_csr(row_ptr, cols, vals, init, tol):
    c = np.array(init, np.float64)
    e = ctypes.c_double()
    conv = lib().orc_davidson_csr(len(row_ptr) - 1, np.ascontiguousarray(row_ptr, np.uint64),
                                  np.ascontiguousarray(cols, np.uint32),
                                  np.ascontiguousarray(vals, np.float64), c, tol, ctypes.byref(e))
    return e.value, c, bool(conv)
