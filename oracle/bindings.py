"""ctypes bindings for the test-only checkers in this directory.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg. The product package never imports this module.

* ``Oracle``: the C restatement of the reference integrand
  (_build/libcdet_oracle.so, built from cdet_oracle.c).
* ``Reference``: the reference's own headers compiled with the quad-precision
  Boost stand-in (_ref/libcdet_ref.so). Available only where the reference
  checkout exists at build time; used to generate and check golden vectors.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libcdet_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libcdet_ref.so")

_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int32)


def build(reference: Optional[str] = None) -> None:
    """Compile the C oracle, and the reference harness when a checkout is given."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if reference and os.path.isdir(os.path.join(reference, "include", "cdet")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFERENCE={reference}"], check=True)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_DP)


class OracleScalars(C.Structure):
    _fields_ = [("n1", C.c_int32), ("n2", C.c_int32), ("cheb_nu", C.c_int32),
                ("cheb_nv", C.c_int32), ("beta", C.c_double), ("u", C.c_double),
                ("branch_eps", C.c_double), ("scale", C.c_double),
                ("diag_up_shift", C.c_double), ("diag_down_shift", C.c_double),
                ("tol_fpm", C.c_double), ("fpm_shift", C.c_double),
                ("z_eps0", C.c_double), ("z_safety", C.c_double)]


class OracleTable(C.Structure):
    _fields_ = [("upper_coeffs", _DP), ("lower_coeffs", _DP),
                ("upper_corners", _DP), ("lower_corners", _DP)]


class OracleTables(C.Structure):
    _fields_ = [("twisted_up", OracleTable), ("twisted_down", OracleTable),
                ("ordinary_up", OracleTable), ("ordinary_down", OracleTable)]


KINDS = ("twisted_up", "twisted_down", "ordinary_up", "ordinary_down")


def _as_numpy_table(t: Dict) -> Dict[str, np.ndarray]:
    out = {}
    for key in ("upper", "lower", "upper_corners", "lower_corners"):
        v = t[key]
        if hasattr(v, "detach"):
            v = v.detach().cpu().numpy()
        out[key] = np.ascontiguousarray(v, dtype=np.float64)
    return out


class Oracle:
    """The C restatement. ``tables`` maps the four kinds to dicts with keys
    upper, lower, upper_corners, lower_corners (numpy or torch float64)."""

    def __init__(self, scalars: dict, tables: Dict[str, Dict]):
        if not os.path.exists(ORACLE_SO):
            build()
        self.lib = lib = C.CDLL(ORACLE_SO)
        lib.oracle_integrand.argtypes = [C.c_void_p, C.c_void_p, _DP, C.c_int, _DP]
        lib.oracle_all_subsets.argtypes = [C.c_void_p, C.c_void_p, _DP, C.c_int, _DP]
        lib.oracle_integrand_batch.argtypes = [C.c_void_p, C.c_void_p, _DP, _IP, C.c_int64,
                                               C.c_int, _DP, _IP, C.c_int]
        lib.oracle_all_subsets_batch.argtypes = [C.c_void_p, C.c_void_p, _DP, C.c_int,
                                                 C.c_int64, _DP, _IP, C.c_int]
        lib.oracle_integrand_ld_batch.argtypes = [C.c_void_p, C.c_void_p, _DP, _IP, C.c_int64,
                                                  C.c_int, _DP, _IP, C.c_int]
        lib.oracle_integrand_ld_parts_batch.argtypes = [C.c_void_p, C.c_void_p, _DP, _IP, C.c_int64,
                                                        C.c_int, _DP, _DP, _IP, C.c_int]
        lib.oracle_mat2pm.argtypes = [_DP, C.c_int, C.c_double, C.c_double, _DP]
        lib.oracle_minors_by_lu.argtypes = [_DP, C.c_int, _DP]
        lib.oracle_ztransform.argtypes = [_DP, _DP, C.c_int, C.c_double, C.c_double]
        lib.oracle_ztransform.restype = C.c_double
        lib.oracle_ztransform_all.argtypes = [_DP, _DP, C.c_int, C.c_double, C.c_double, _DP]
        lib.oracle_fill_green.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, _DP, C.c_int,
                                          C.c_int, _DP, _DP, _DP, _DP]
        lib.oracle_prefactor_dd.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _DP, _DP]
        lib.oracle_prefactor_ld.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
        lib.oracle_prefactor_ld.restype = C.c_double
        lib.oracle_diagonal_order1.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, _DP]
        _UP = C.POINTER(C.c_uint64)
        lib.oracle_mcmcmc_chain.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, _DP, C.c_int,
                                            C.c_int, C.c_double, C.c_int, C.c_uint64, _UP, _DP, _DP, _DP, _DP,
                                            _UP]
        lib.oracle_mcmcmc_chain_hist.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, _DP, C.c_int,
                                                 C.c_int, C.c_double, C.c_int, C.c_uint64, C.c_int, _DP, _DP, _DP,
                                                 _UP, _DP, _DP, _DP, _DP, _UP]
        lib.oracle_learn_histogram.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                               C.c_int, C.c_double, C.c_double, C.c_uint64, _DP, _DP, _DP, _DP]
        self.scalars = OracleScalars(**{k: scalars[k] for k, _ in OracleScalars._fields_})
        self._keep = {k: _as_numpy_table(tables[k]) for k in KINDS}
        tabs = {}
        for k in KINDS:
            t = self._keep[k]
            tabs[k] = OracleTable(_ptr(t["upper"]), _ptr(t["lower"]),
                                  _ptr(t["upper_corners"]), _ptr(t["lower_corners"]))
        self.tables = OracleTables(**tabs)

    def integrand(self, vertices: np.ndarray) -> tuple:
        v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 4)
        out = C.c_double()
        st = self.lib.oracle_integrand(C.byref(self.scalars), C.byref(self.tables), _ptr(v),
                                       v.shape[0], C.byref(out))
        return out.value, st

    def all_subsets(self, vertices: np.ndarray) -> tuple:
        v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 4)
        out = np.zeros(1 << v.shape[0])
        st = self.lib.oracle_all_subsets(C.byref(self.scalars), C.byref(self.tables), _ptr(v),
                                         v.shape[0], _ptr(out))
        return out, st

    def integrand_batch(self, vertices: np.ndarray, orders: np.ndarray, threads: int = 1):
        v = np.ascontiguousarray(vertices, dtype=np.float64)
        o = np.ascontiguousarray(orders, dtype=np.int32)
        batch, max_order = v.shape[0], v.shape[1]
        out = np.zeros(batch)
        st = np.zeros(batch, dtype=np.int32)
        rc = self.lib.oracle_integrand_batch(C.byref(self.scalars), C.byref(self.tables),
                                             _ptr(v), o.ctypes.data_as(_IP), batch, max_order,
                                             _ptr(out), st.ctypes.data_as(_IP), threads)
        if rc != 0:
            raise RuntimeError("oracle thread start failed")
        return out, st

    def integrand_ld_batch(self, vertices: np.ndarray, orders: np.ndarray, threads: int = 1):
        """The long double truth of each configuration's integrand (rounded
        to double), for error measurements; see oracle_integrand_ld."""
        v = np.ascontiguousarray(vertices, dtype=np.float64)
        o = np.ascontiguousarray(orders, dtype=np.int32)
        batch, max_order = v.shape[0], v.shape[1]
        out = np.zeros(batch)
        st = np.zeros(batch, dtype=np.int32)
        rc = self.lib.oracle_integrand_ld_batch(C.byref(self.scalars), C.byref(self.tables),
                                                _ptr(v), o.ctypes.data_as(_IP), batch, max_order,
                                                _ptr(out), st.ctypes.data_as(_IP), threads)
        if rc != 0:
            raise RuntimeError("oracle thread start failed")
        return out, st

    def integrand_ld_parts_batch(self, vertices: np.ndarray, orders: np.ndarray, threads: int = 1):
        """The long double truth with its parts: returns (values [batch],
        parts [batch][4] = twisted, ordinary, twisted magnitude, ordinary
        magnitude (see oracle_integrand_ld_parts), status [batch])."""
        v = np.ascontiguousarray(vertices, dtype=np.float64)
        o = np.ascontiguousarray(orders, dtype=np.int32)
        batch, max_order = v.shape[0], v.shape[1]
        out = np.zeros(batch)
        parts = np.zeros((batch, 4))
        st = np.zeros(batch, dtype=np.int32)
        rc = self.lib.oracle_integrand_ld_parts_batch(C.byref(self.scalars), C.byref(self.tables),
                                                      _ptr(v), o.ctypes.data_as(_IP), batch, max_order,
                                                      _ptr(out), _ptr(parts), st.ctypes.data_as(_IP), threads)
        if rc != 0:
            raise RuntimeError("oracle thread start failed")
        return out, parts, st

    def all_subsets_batch(self, vertices: np.ndarray, threads: int = 1):
        v = np.ascontiguousarray(vertices, dtype=np.float64)
        batch, env = v.shape[0], v.shape[1]
        out = np.zeros((batch, 1 << env))
        st = np.zeros(batch, dtype=np.int32)
        rc = self.lib.oracle_all_subsets_batch(C.byref(self.scalars), C.byref(self.tables),
                                               _ptr(v), env, batch, _ptr(out),
                                               st.ctypes.data_as(_IP), threads)
        if rc != 0:
            raise RuntimeError("oracle thread start failed")
        return out, st

    def green(self, vertices: np.ndarray, replica_count: int, twisted: bool):
        v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 4)
        n = v.shape[0]
        mu, md = np.zeros(n * n), np.zeros(n * n)
        du, dd = np.zeros(n), np.zeros(n)
        tu = self.tables.twisted_up if twisted else self.tables.ordinary_up
        td = self.tables.twisted_down if twisted else self.tables.ordinary_down
        st = self.lib.oracle_fill_green(C.byref(self.scalars), C.byref(tu), C.byref(td), _ptr(v),
                                        n, replica_count, _ptr(mu), _ptr(md), _ptr(du), _ptr(dd))
        return mu.reshape(n, n), md.reshape(n, n), du, dd, st

    def diagonal_order1(self, alpha_up: float, alpha_down: float) -> np.ndarray:
        """[twisted - 2 ordinary, twisted, ordinary] order-1 diagonal densities."""
        out = np.zeros(3)
        rc = self.lib.oracle_diagonal_order1(C.byref(self.scalars), C.byref(self.tables),
                                             float(alpha_up), float(alpha_down), _ptr(out))
        if rc != 0:
            raise RuntimeError("The diagonal observable is undefined for U = 0")
        return out

    def mcmcmc_chain(self, order_min, order_max, envelope, lambdas, warmup, adapt_interval,
                     adapt_rate, production, seed, histogram=None):
        """One chain with the uniform seed kernel, or the histogram seed of
        histogram = (tau_bins, tau, space, replica); the same outputs as
        Reference.mcmcmc_chain."""
        steps = warmup + production
        chosen = np.zeros(steps, dtype=np.uint64)
        norms = np.zeros(steps)
        signal = np.zeros((production, envelope + 1))
        verts = np.zeros((envelope, 4))
        lam = np.ascontiguousarray(lambdas, dtype=np.float64)
        lam_out = np.zeros(envelope + 1)
        rng = np.zeros(8, dtype=np.uint64)
        up = C.POINTER(C.c_uint64)
        if histogram is None:
            rc = self.lib.oracle_mcmcmc_chain(C.byref(self.scalars), C.byref(self.tables), order_min, order_max,
                                              envelope, _ptr(lam), warmup, adapt_interval, adapt_rate, production,
                                              seed, chosen.ctypes.data_as(up), _ptr(norms), _ptr(signal),
                                              _ptr(verts), _ptr(lam_out), rng.ctypes.data_as(up))
        else:
            bins, ht, hs, hr = histogram
            ht, hs, hr = (np.ascontiguousarray(x, dtype=np.float64) for x in (ht, hs, hr))
            rc = self.lib.oracle_mcmcmc_chain_hist(C.byref(self.scalars), C.byref(self.tables), order_min,
                                                   order_max, envelope, _ptr(lam), warmup, adapt_interval,
                                                   adapt_rate, production, seed, bins, _ptr(ht), _ptr(hs),
                                                   _ptr(hr), chosen.ctypes.data_as(up), _ptr(norms),
                                                   _ptr(signal), _ptr(verts), _ptr(lam_out),
                                                   rng.ctypes.data_as(up))
        if rc != 0:
            raise RuntimeError(f"oracle chain failed ({rc})")
        return dict(chosen=chosen, norms=norms, signal=signal, vertices=verts, lambdas=lam_out, rng=rng)

    def learn_histogram(self, order_min, order_max, envelope, learning_steps, tau_bins, uniform_mix,
                        pseudo_count, base_seed):
        """learn_factorized_histogram_seed: (tau, space, replica, total pair weight)."""
        sites = self.scalars.n1 * self.scalars.n2
        tau, space, rep = np.zeros(tau_bins * tau_bins), np.zeros(sites * sites), np.zeros(4)
        total = C.c_double()
        rc = self.lib.oracle_learn_histogram(C.byref(self.scalars), C.byref(self.tables), order_min, order_max,
                                             envelope, learning_steps, tau_bins, uniform_mix, pseudo_count,
                                             base_seed, _ptr(tau), _ptr(space), _ptr(rep), C.byref(total))
        if rc != 0:
            raise RuntimeError(f"oracle histogram learning failed ({rc})")
        return tau, space, rep, total.value

    @staticmethod
    def _lib():
        if not os.path.exists(ORACLE_SO):
            build()
        lib = C.CDLL(ORACLE_SO)
        lib.oracle_mat2pm.argtypes = [_DP, C.c_int, C.c_double, C.c_double, _DP]
        lib.oracle_minors_by_lu.argtypes = [_DP, C.c_int, _DP]
        lib.oracle_ztransform.argtypes = [_DP, _DP, C.c_int, C.c_double, C.c_double]
        lib.oracle_ztransform.restype = C.c_double
        lib.oracle_ztransform_all.argtypes = [_DP, _DP, C.c_int, C.c_double, C.c_double, _DP]
        lib.oracle_prefactor_dd.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _DP, _DP]
        lib.oracle_prefactor_ld.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
        lib.oracle_prefactor_ld.restype = C.c_double
        return lib


def oracle_mat2pm(a: np.ndarray, tol: float, shift: float):
    lib = Oracle._lib()
    a = np.ascontiguousarray(a, dtype=np.float64)
    n = a.shape[0]
    out = np.zeros((1 << n) - 1)
    fell_back = lib.oracle_mat2pm(_ptr(a), n, tol, shift, _ptr(out))
    return out, fell_back


def oracle_minors_by_lu(a: np.ndarray):
    lib = Oracle._lib()
    a = np.ascontiguousarray(a, dtype=np.float64)
    n = a.shape[0]
    out = np.zeros((1 << n) - 1)
    lib.oracle_minors_by_lu(_ptr(a), n, _ptr(out))
    return out


def oracle_ztransform(up, down, n, eps0, safety):
    lib = Oracle._lib()
    up = np.ascontiguousarray(up, dtype=np.float64)
    down = np.ascontiguousarray(down, dtype=np.float64)
    return lib.oracle_ztransform(_ptr(up), _ptr(down), n, eps0, safety)


def oracle_ztransform_all(up, down, n, eps0, safety):
    lib = Oracle._lib()
    up = np.ascontiguousarray(up, dtype=np.float64)
    down = np.ascontiguousarray(down, dtype=np.float64)
    out = np.zeros(1 << n)
    lib.oracle_ztransform_all(_ptr(up), _ptr(down), n, eps0, safety, _ptr(out))
    return out


def oracle_prefactors(order, n1, n2, replica_count):
    lib = Oracle._lib()
    hi, lo = C.c_double(), C.c_double()
    lib.oracle_prefactor_dd(order, n1, n2, replica_count, C.byref(hi), C.byref(lo))
    return hi.value, lo.value, lib.oracle_prefactor_ld(order, n1, n2, replica_count)


class Reference:
    """The reference's own integrand, compiled here (oracle/_ref)."""

    def __init__(self):
        if not os.path.exists(REF_SO):
            raise FileNotFoundError(REF_SO)
        self.lib = lib = C.CDLL(REF_SO)
        lib.ref_last_error.restype = C.c_char_p
        lib.ref_configure.argtypes = [C.c_int, C.c_int] + [C.c_char_p] * 5 + \
            [C.c_int, C.c_char_p, C.c_int, C.c_int, C.c_int] + [C.c_char_p] * 5
        lib.ref_set_precision.argtypes = [C.c_char_p, C.c_char_p]
        lib.ref_build_tables.argtypes = [C.c_int]
        lib.ref_coeff_count.restype = C.c_size_t
        lib.ref_corner_count.restype = C.c_size_t
        lib.ref_get_table.argtypes = [C.c_int, _DP, _DP, _DP, _DP]
        lib.ref_set_table.argtypes = [C.c_int, _DP, _DP, _DP, _DP]
        lib.ref_set_table_long_double.argtypes = [C.c_int, _DP, _DP, _DP, _DP]
        lib.ref_eval_integrand.argtypes = [_DP, C.c_int, _DP]
        lib.ref_eval_integrand_batch.argtypes = [_DP, C.POINTER(C.c_int), C.c_int, C.c_int, _DP,
                                                 C.c_int]
        lib.ref_eval_all_subsets.argtypes = [_DP, C.c_int, _DP]
        lib.ref_mat2pm.argtypes = [_DP, C.c_int, C.c_double, C.c_double, _DP]
        lib.ref_minors_by_lu.argtypes = [_DP, C.c_int, _DP]
        lib.ref_ztransform.argtypes = [_DP, _DP, C.c_int, C.c_double, C.c_double]
        lib.ref_ztransform.restype = C.c_double
        lib.ref_ztransform_all.argtypes = [_DP, _DP, C.c_int, C.c_double, C.c_double, _DP]
        lib.ref_lookup_descriptor.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double] + \
            [C.c_int] * 4 + [C.c_double, C.c_double] + [C.c_int] * 5 + \
            [C.POINTER(C.c_int), C.POINTER(C.c_ulonglong), _DP, _DP]
        lib.ref_green_replica.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                          C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                          C.c_double, C.c_int, _DP]
        lib.ref_fpm_fallbacks.restype = C.c_ulonglong
        lib.ref_sample_vertices.argtypes = [C.c_ulonglong, C.c_int, _DP]
        lib.ref_diagonal_order1.argtypes = [_DP]
        lib.ref_chunk_workflow.argtypes = [C.c_char_p, C.c_int, C.c_int]
        lib.ref_load_chunks.argtypes = [C.c_char_p]
        _UP = C.POINTER(C.c_ulonglong)
        lib.ref_mcmcmc_chain.argtypes = [C.c_int, C.c_int, C.c_int, _DP, C.c_int, C.c_int, C.c_double,
                                         C.c_int, C.c_ulonglong, C.c_int, _DP, _DP, _DP, _UP, _DP, _DP, _DP,
                                         _DP, _UP]
        lib.ref_learn_histogram.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                            C.c_double, C.c_ulonglong, _DP, _DP, _DP, _DP]
        lib.ref_mcmcmc_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _DP, C.c_int, C.c_int, C.c_double,
                                       C.c_int, C.c_int, C.c_ulonglong, C.c_int, _DP, _DP, _DP, C.c_char_p,
                                       C.c_ulonglong, C.c_char_p, _UP, _DP, _DP, _DP, _DP]

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(self.lib.ref_last_error().decode())

    def configure(self, n1, n2, beta, mu, u, alpha_up, alpha_down, pbc, mask_name, radius,
                  nu, nv, branch_eps="1e-13", tol_fpm="1e-7", fpm_shift="auto",
                  z_eps0="auto", z_safety="1e4"):
        e = lambda s: str(s).encode()
        self._check(self.lib.ref_configure(n1, n2, e(beta), e(mu), e(u), e(alpha_up),
                                           e(alpha_down), int(pbc), e(mask_name), radius, nu, nv,
                                           e(branch_eps), e(tol_fpm), e(fpm_shift), e(z_eps0),
                                           e(z_safety)))

    def build_tables(self, threads: int = 4):
        self._check(self.lib.ref_build_tables(threads))

    def set_precision(self, vector_real: str, integrand_real: str) -> None:
        """VECTOR_REAL / INTEGRAND_REAL of later evaluations (precision_config.h:15-26)."""
        self._check(self.lib.ref_set_precision(vector_real.encode(), integrand_real.encode()))

    def get_tables(self) -> Dict[str, Dict[str, np.ndarray]]:
        nc, nk = self.lib.ref_coeff_count(), self.lib.ref_corner_count()
        out = {}
        for i, kind in enumerate(KINDS):
            t = {"upper": np.zeros(nc), "lower": np.zeros(nc),
                 "upper_corners": np.zeros(nk), "lower_corners": np.zeros(nk)}
            self._check(self.lib.ref_get_table(i, _ptr(t["upper"]), _ptr(t["lower"]),
                                               _ptr(t["upper_corners"]),
                                               _ptr(t["lower_corners"])))
            out[kind] = t
        return out

    def set_tables(self, tables: Dict[str, Dict], long_double: bool = False):
        """Resident tables (double; or widened to long double for
        VECTOR_REAL=long_double)."""
        setter = self.lib.ref_set_table_long_double if long_double else self.lib.ref_set_table
        for i, kind in enumerate(KINDS):
            t = _as_numpy_table(tables[kind])
            self._check(setter(i, _ptr(t["upper"]), _ptr(t["lower"]), _ptr(t["upper_corners"]),
                               _ptr(t["lower_corners"])))

    def integrand(self, vertices) -> float:
        v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 4)
        out = C.c_double()
        self._check(self.lib.ref_eval_integrand(_ptr(v), v.shape[0], C.byref(out)))
        return out.value

    def integrand_batch(self, vertices: np.ndarray, orders: np.ndarray, threads: int = 1):
        v = np.ascontiguousarray(vertices, dtype=np.float64)
        o = np.ascontiguousarray(orders, dtype=np.int32)
        out = np.zeros(v.shape[0])
        fails = self.lib.ref_eval_integrand_batch(_ptr(v), o.ctypes.data_as(C.POINTER(C.c_int)),
                                                  v.shape[0], v.shape[1], _ptr(out), threads)
        return out, fails

    def all_subsets(self, vertices) -> np.ndarray:
        v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 4)
        out = np.zeros(1 << v.shape[0])
        self._check(self.lib.ref_eval_all_subsets(_ptr(v), v.shape[0], _ptr(out)))
        return out

    def mcmcmc_chain(self, order_min, order_max, envelope, lambdas, warmup, adapt_interval,
                     adapt_rate, production, seed, histogram=None):
        """One reference chain (uniform seed, or the FactorizedHistogramSeed of
        histogram = (tau_bins, tau, space, replica)): per-step chosen masks and
        local normalisations, production order signals, final vertices,
        lambdas and the next 8 raw generator outputs."""
        steps = warmup + production
        chosen = np.zeros(steps, dtype=np.uint64)
        norms = np.zeros(steps)
        signal = np.zeros((production, envelope + 1))
        verts = np.zeros((envelope, 4))
        lam = np.ascontiguousarray(lambdas, dtype=np.float64)
        lam_out = np.zeros(envelope + 1)
        rng = np.zeros(8, dtype=np.uint64)
        up = C.POINTER(C.c_ulonglong)
        bins, ht, hs, hr = (0, np.zeros(1), np.zeros(1), np.zeros(1)) if histogram is None else histogram
        ht, hs, hr = (np.ascontiguousarray(x, dtype=np.float64) for x in (ht, hs, hr))
        self._check(self.lib.ref_mcmcmc_chain(order_min, order_max, envelope, _ptr(lam), warmup,
                                              adapt_interval, adapt_rate, production, seed, bins, _ptr(ht),
                                              _ptr(hs), _ptr(hr), chosen.ctypes.data_as(up), _ptr(norms),
                                              _ptr(signal), _ptr(verts), _ptr(lam_out), rng.ctypes.data_as(up)))
        return dict(chosen=chosen, norms=norms, signal=signal, vertices=verts, lambdas=lam_out, rng=rng)

    def learn_histogram(self, order_min, order_max, envelope, learning_steps, tau_bins, uniform_mix,
                        pseudo_count, base_seed, sites):
        """learn_factorized_histogram_seed: (tau, space, replica) row
        probabilities and the total pair weight."""
        tau = np.zeros(tau_bins * tau_bins)
        space = np.zeros(sites * sites)
        rep = np.zeros(4)
        total = C.c_double()
        self._check(self.lib.ref_learn_histogram(order_min, order_max, envelope, learning_steps, tau_bins,
                                                 uniform_mix, pseudo_count, base_seed, _ptr(tau), _ptr(space),
                                                 _ptr(rep), C.byref(total)))
        return tau, space, rep, total.value

    def mcmcmc_run(self, order_min, order_max, envelope, normalization_order, lambdas, warmup, adapt_interval,
                   adapt_rate, production, chains, base_seed, histogram=None, checkpoint_dir="",
                   checkpoint_interval=10_000_000, resume_mode="off"):
        """run_mcmcmc_chains_parallel: per-chain results (u64 [chains][5 + 2(env+1)],
        stats [chains][3 + env][5] as (count, mean hi, lo, m2 hi, lo)), final
        lambdas, cross-chain stats [env+1][5] and ratios [env+1][2] (hi, lo)."""
        e1 = envelope + 1
        u64 = np.zeros((chains, 5 + 2 * e1), dtype=np.uint64)
        stats = np.zeros((chains, 2 + e1, 5))
        lam_out = np.zeros((chains, e1))
        cross = np.zeros((e1, 5))
        ratios = np.zeros((e1, 2))
        lam = np.ascontiguousarray(lambdas, dtype=np.float64)
        bins, ht, hs, hr = (0, np.zeros(1), np.zeros(1), np.zeros(1)) if histogram is None else histogram
        ht, hs, hr = (np.ascontiguousarray(x, dtype=np.float64) for x in (ht, hs, hr))
        self._check(self.lib.ref_mcmcmc_run(order_min, order_max, envelope, normalization_order, _ptr(lam), warmup,
                                            adapt_interval, adapt_rate, production, chains, base_seed, bins,
                                            _ptr(ht), _ptr(hs), _ptr(hr), checkpoint_dir.encode(),
                                            checkpoint_interval, resume_mode.encode(),
                                            u64.ctypes.data_as(C.POINTER(C.c_ulonglong)), _ptr(stats),
                                            _ptr(lam_out), _ptr(cross), _ptr(ratios)))
        return dict(u64=u64, stats=stats, lambdas=lam_out, cross=cross, ratios=ratios)

    def chunk_workflow(self, directory: str, node_chunk_size: int, sitepair_chunk_size: int) -> None:
        """Runs every stage of the reference's chunked load-data workflow into
        `directory` for the configured parameter set."""
        self._check(self.lib.ref_chunk_workflow(directory.encode(), node_chunk_size, sitepair_chunk_size))

    def load_chunks(self, directory: str) -> None:
        """load_chunked_data_into_resident_tables from `directory`."""
        self._check(self.lib.ref_load_chunks(directory.encode()))

    def diagonal_order1(self) -> np.ndarray:
        """[normalised hi, twisted, ordinary, normalised lo] from the reference."""
        out = np.zeros(4)
        self._check(self.lib.ref_diagonal_order1(_ptr(out)))
        return out

    def mat2pm(self, a, tol, shift):
        a = np.ascontiguousarray(a, dtype=np.float64)
        out = np.zeros((1 << a.shape[0]) - 1)
        self._check(self.lib.ref_mat2pm(_ptr(a), a.shape[0], tol, shift, _ptr(out)))
        return out

    def minors_by_lu(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        out = np.zeros((1 << a.shape[0]) - 1)
        self._check(self.lib.ref_minors_by_lu(_ptr(a), a.shape[0], _ptr(out)))
        return out

    def ztransform(self, up, down, n, eps0, safety):
        up = np.ascontiguousarray(up, dtype=np.float64)
        down = np.ascontiguousarray(down, dtype=np.float64)
        return self.lib.ref_ztransform(_ptr(up), _ptr(down), n, eps0, safety)

    def ztransform_all(self, up, down, n, eps0, safety):
        up = np.ascontiguousarray(up, dtype=np.float64)
        down = np.ascontiguousarray(down, dtype=np.float64)
        out = np.zeros(1 << n)
        self._check(self.lib.ref_ztransform_all(_ptr(up), _ptr(down), n, eps0, safety, _ptr(out)))
        return out

    def lookup_descriptor(self, ra, rb, tau1, tau2, x1, y1, x2, y2, beta, eps, nu, nv, n1, n2,
                          upper):
        corner, index = C.c_int(), C.c_ulonglong()
        u, v = C.c_double(), C.c_double()
        self._check(self.lib.ref_lookup_descriptor(ra, rb, tau1, tau2, x1, y1, x2, y2, beta, eps,
                                                   nu, nv, n1, n2, int(upper), C.byref(corner),
                                                   C.byref(index), C.byref(u), C.byref(v)))
        return corner.value, index.value, u.value, v.value

    def green_replica(self, n1, n2, beta, mu, pbc, mask_name, radius, ra, rb, tau, tau_p, upper):
        out = np.zeros((n1 * n2) ** 2)
        self._check(self.lib.ref_green_replica(n1, n2, beta, mu, int(pbc), mask_name.encode(),
                                               radius, ra, rb, tau, tau_p, int(upper), _ptr(out)))
        return out.reshape(n1 * n2, n1 * n2)

    def fpm_fallbacks(self) -> int:
        return self.lib.ref_fpm_fallbacks()

    def sample_vertices(self, seed: int, count: int) -> np.ndarray:
        out = np.zeros(count * 4)
        self.lib.ref_sample_vertices(seed, count, _ptr(out))
        return out.reshape(count, 4)
