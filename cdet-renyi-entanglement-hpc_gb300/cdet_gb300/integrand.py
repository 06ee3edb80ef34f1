"""Host-side mirror of the reference integrand interface, on the GB300 kernels.

``CdetIntegrand`` holds one parameter set and its four resident tables in HBM
and exposes the reference's two entry points with the reference's names,
argument meaning and errors:

* ``evaluate_cdet_density_integrand_double(vertices)``
  (cdet_integrand_evaluator.h:542-560)
* ``evaluate_cdet_density_all_subset_integrands_double_into(vertices, values)``
  (:562-583) and the by-value form (:585-590)

plus batched forms on host or device buffers, which the C ABI
(include/cdet_gb300.h) provides and which a driver that evaluates many
proposals per step calls instead of one configuration at a time.
"""
from __future__ import annotations

import ctypes as C
import os
from collections import namedtuple
from typing import Dict, Iterable, List, Optional, Sequence

import numpy as np

from . import lib as L
from .params import CdetParams

# UnitVertex (cdet_integrand_evaluator.h:16-21): tau, x, y, replica in [0, 1).
UnitVertex = namedtuple("UnitVertex", ["tau", "x", "y", "replica"])


def _as_vertex_array(vertices) -> np.ndarray:
    if isinstance(vertices, np.ndarray):
        arr = vertices
    else:
        arr = np.array([[v.tau, v.x, v.y, v.replica] if isinstance(v, UnitVertex) else list(v)
                        for v in vertices], dtype=np.float64)
    return np.ascontiguousarray(arr, dtype=np.float64).reshape(-1, 4)


def _ptr(obj) -> int:
    """Address of a numpy array or a torch tensor (host or device)."""
    if hasattr(obj, "data_ptr"):
        return obj.data_ptr()
    return obj.ctypes.data


class CdetIntegrand:
    """The CDet integrand of one parameter set on one CUDA device.

    ``tables`` maps the four kinds (twisted_up, twisted_down, ordinary_up,
    ordinary_down) to dicts with float64 arrays ``upper``, ``lower``,
    ``upper_corners``, ``lower_corners``. CUDA torch tensors are used in place
    (the caller keeps them alive); numpy arrays and CPU tensors are copied to
    HBM. Kinds whose dict is the same object as another kind's are aliased, as
    the reference does when ALPHA_UP == ALPHA_DOWN.
    """

    def __init__(self, params: CdetParams, tables: Optional[Dict[str, Dict]], device: int = 0):
        self.params = params
        self._assembly = "fp64"
        self.scalars = params.runtime_scalars()
        self._lib = L.load()
        self._ctx = C.c_void_p()
        rs = L.RuntimeScalars(**{k: self.scalars[k] for k, _ in L.RuntimeScalars._fields_})
        L.check(self._lib.cdet_create(C.byref(rs), device, C.byref(self._ctx)))
        self._keep = []
        sites = params.sites
        self.coeff_count = 4 * sites * sites * params.cheb_nu * params.cheb_nv
        self.corner_count = 4 * sites * sites
        seen = {}
        for kind, name in enumerate(L.KIND_NAMES if tables is not None else ()):
            t = tables[name]
            if id(t) in seen:
                L.check(self._lib.cdet_alias_table(self._ctx, kind, seen[id(t)]))
                continue
            seen[id(t)] = kind
            self._set_table(kind, t)

    def _set_table(self, kind: int, t: Dict) -> None:
        arrays = [t["upper"], t["lower"], t["upper_corners"], t["lower_corners"]]
        on_device = all(hasattr(a, "is_cuda") and a.is_cuda for a in arrays)
        if on_device:
            for a in arrays:
                if a.dtype.__str__() != "torch.float64" or not a.is_contiguous():
                    raise ValueError("device tables must be contiguous float64 tensors")
            self._keep.append(arrays)
            view = L.TableView(*[a.data_ptr() for a in arrays])
            L.check(self._lib.cdet_bind_device_table(self._ctx, kind, C.byref(view),
                                                     self.coeff_count, self.corner_count))
        else:
            host = [np.ascontiguousarray(a.detach().cpu().numpy() if hasattr(a, "detach") else a,
                                         dtype=np.float64) for a in arrays]
            view = L.TableView(*[h.ctypes.data for h in host])
            L.check(self._lib.cdet_upload_table(self._ctx, kind, C.byref(view),
                                                self.coeff_count, self.corner_count))

    def load_chunks(self, directory: str) -> Optional[tuple]:
        """Loads the four tables from a chunked load-data directory of the
        reference's chunk workflow straight into HBM
        (load_chunked_data_into_resident_tables, chunked_load_data.h:1467-1479).
        Returns the directory's precomputed diagonal order-1 value (hi, lo),
        or None when it has none."""
        out = np.zeros(2)
        L.check(self._lib.cdet_load_chunks(self._ctx, os.fsencode(directory),
                                           out.ctypes.data_as(C.POINTER(C.c_double))))
        self._keep = []
        return None if np.isnan(out[0]) else (float(out[0]), float(out[1]))

    def close(self) -> None:
        if self._ctx:
            self._lib.cdet_destroy(self._ctx)
            self._ctx = C.c_void_p()
            self._keep = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ batched ---
    def reserve(self, batch: int, max_order: int) -> None:
        L.check(self._lib.cdet_reserve(self._ctx, int(batch), int(max_order)))

    def integrand_batch(self, vertices: np.ndarray, orders: Sequence[int], check: bool = False):
        """Host buffers: vertices [batch][max_order][4], orders [batch].
        Returns (values [batch], status [batch])."""
        v = np.ascontiguousarray(vertices, dtype=np.float64)
        o = np.ascontiguousarray(orders, dtype=np.int32)
        batch, max_order = v.shape[0], v.shape[1]
        values = np.zeros(batch)
        status = np.zeros(batch, dtype=np.int32)
        rc = self._lib.cdet_integrand_host(self._ctx, v.ctypes.data, o.ctypes.data, batch,
                                           max_order, values.ctypes.data, status.ctypes.data)
        if rc not in (L.CDET_OK, L.CDET_ERR_VALUE) or (check and rc != L.CDET_OK):
            L.check(rc)
        return values, status

    def all_subsets_batch(self, vertices: np.ndarray, check: bool = False):
        """Host buffers: vertices [batch][envelope][4]. Returns
        (values [batch][2^envelope], status [batch])."""
        v = np.ascontiguousarray(vertices, dtype=np.float64)
        batch, env = v.shape[0], v.shape[1]
        values = np.zeros((batch, 1 << env))
        status = np.zeros(batch, dtype=np.int32)
        rc = self._lib.cdet_all_subsets_host(self._ctx, v.ctypes.data, env, batch,
                                             values.ctypes.data, status.ctypes.data)
        if rc not in (L.CDET_OK, L.CDET_ERR_VALUE) or (check and rc != L.CDET_OK):
            L.check(rc)
        return values, status

    def integrand_device(self, vertices, orders, values, status, stream=None) -> None:
        """Device buffers (torch CUDA tensors or raw addresses), asynchronous
        on ``stream`` (a torch.cuda.Stream, a cudaStream_t address or None)."""
        batch, max_order = int(vertices.shape[0]), int(vertices.shape[1])
        L.check(self._lib.cdet_integrand_device(self._ctx, _ptr(vertices), _ptr(orders), batch,
                                                max_order, _ptr(values), _ptr(status),
                                                _stream_handle(stream)))

    def integrand_device_noalloc(self, vertices, orders, values, status, stream=None) -> int:
        """cdet_integrand_device_noalloc: the FP64 form on the library's fixed
        static scratch, allocating no device memory. Returns the C-ABI code
        (0 on success); the message of a failure is in lib.last_error()."""
        batch, max_order = int(vertices.shape[0]), int(vertices.shape[1])
        return int(self._lib.cdet_integrand_device_noalloc(self._ctx, _ptr(vertices), _ptr(orders), batch,
                                                           max_order, _ptr(values), _ptr(status),
                                                           _stream_handle(stream)))

    def all_subsets_device(self, vertices, values, status, stream=None) -> None:
        batch, env = int(vertices.shape[0]), int(vertices.shape[1])
        L.check(self._lib.cdet_all_subsets_device(self._ctx, _ptr(vertices), env, batch,
                                                  _ptr(values), _ptr(status),
                                                  _stream_handle(stream)))

    def counters(self):
        calls, fallbacks = C.c_uint64(), C.c_uint64()
        L.check(self._lib.cdet_counters(self._ctx, C.byref(calls), C.byref(fallbacks)))
        return calls.value, fallbacks.value

    def diagonal_order1_density(self) -> np.ndarray:
        """Deterministic order-1 diagonal observable of the bound tables,
        [twisted - 2 ordinary, twisted, ordinary]
        (diagonal_green_observable.h:237-366), bit-identical to the reference."""
        out = np.zeros(3)
        L.check(self._lib.cdet_diagonal_order1_density(self._ctx, float(self.params.alpha_up),
                                                       float(self.params.alpha_down),
                                                       out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def last_launch_count(self) -> int:
        return int(self._lib.cdet_last_launch_count(self._ctx))

    def set_all_subsets_form(self, form: str) -> None:
        """'auto', 'lane' or 'warp': the work layout of the all-subsets CDet
        recursion (same values bit for bit, different speed)."""
        code = {"auto": 0, "lane": 1, "warp": 2}[form]
        L.check(self._lib.cdet_set_all_subsets_form(self._ctx, code))

    def all_subsets_form_tuned(self, max_order: int, batch: int) -> str:
        """The all-subsets form the autotuner kept for this order and batch
        size class under the current assembly ('auto' before a measurement)."""
        form = C.c_int()
        L.check(self._lib.cdet_all_subsets_form_tuned(self._ctx, int(max_order), int(self._assembly == "split"),
                                                      int(batch), C.byref(form)))
        return {0: "auto", 1: "lane", 2: "warp"}[form.value]

    def set_integrand_form(self, form: str, warps_per_sm: int = 0, pair: bool = False, grab: int = 1) -> None:
        """'auto', 'staged' or 'queue': how a single-top batch of order <= 10
        runs after its Green matrices (same values bit for bit, different
        speed). For 'queue' also the launch shape: resident warps per SM (0:
        as many as shared memory holds), two warps per configuration (pair)
        and the slots a warp takes per queue pop (grab)."""
        code = {"auto": 0, "staged": 1, "queue": 2}[form]
        L.check(self._lib.cdet_set_integrand_form(self._ctx, code, int(warps_per_sm), int(bool(pair)), int(grab)))

    def integrand_form_tuned(self, max_order: int, batch: int) -> dict:
        """The form the autotuner kept for this order and batch size class
        under the current assembly ({'form': 'auto'} before a measurement)."""
        out = [C.c_int() for _ in range(4)]
        L.check(self._lib.cdet_integrand_form_tuned(self._ctx, int(max_order), int(self._assembly == "split"),
                                                    int(batch), *[C.byref(x) for x in out]))
        form = {0: "auto", 1: "staged", 2: "queue"}[out[0].value]
        if form != "queue":
            return {"form": form}
        return {"form": form, "warps_per_sm": out[1].value, "pair": bool(out[2].value), "grab": out[3].value}

    def set_integrand_real(self, real: str, significand_bits: int = 0) -> None:
        """INTEGRAND_REAL: "double" (the FP64 drop-in, default) or
        "double_double" (with VECTOR_REAL=double: the FP64 Green matrices,
        then minors, CDet and the order-1 branch in the reference's
        DoubleDouble arithmetic). significand_bits = 113 takes the parameters'
        DoubleDouble values as a quad-precision MP_Real gives them."""
        from .params import dd_scalars
        if real == "double":
            L.check(self._lib.cdet_set_integrand_real(self._ctx, L.INTEGRAND_REAL_DOUBLE, None))
            return
        if real != "double_double":
            raise ValueError("INTEGRAND_REAL must be double or double_double")
        values = dd_scalars(self.params, significand_bits)
        scalars = L.DDScalars(**{k: L.DD(*v) for k, v in values.items()})
        L.check(self._lib.cdet_set_integrand_real(self._ctx, L.INTEGRAND_REAL_DOUBLE_DOUBLE, C.byref(scalars)))

    def set_assembly(self, mode: str) -> None:
        """"fp64": the reference's Clenshaw in FP64, bit-identical (default);
        "split": batched split-bf16 tcgen05 assembly, FP64-level accuracy."""
        code = {"fp64": L.ASSEMBLY_FP64, "split": L.ASSEMBLY_SPLIT_BF16}[mode]
        L.check(self._lib.cdet_set_assembly(self._ctx, code))
        self._assembly = mode

    def prepare_split(self) -> None:
        """Slice the tables for the split assembly now (device memory)."""
        L.check(self._lib.cdet_prepare_split(self._ctx))

    def assemble(self, vertices, orders, stream=None):
        """Green matrices of the current assembly mode for device (torch)
        inputs: returns (green [batch][2][2][max_order^2],
        diag [batch][2][2][max_order], status)."""
        import torch
        batch, nmax = int(vertices.shape[0]), int(vertices.shape[1])
        green = torch.zeros((batch, 2, 2, nmax * nmax), dtype=torch.float64, device=vertices.device)
        diag = torch.zeros((batch, 2, 2, nmax), dtype=torch.float64, device=vertices.device)
        status = torch.zeros(batch, dtype=torch.int32, device=vertices.device)
        L.check(self._lib.cdet_assemble_device(self._ctx, _ptr(vertices), _ptr(orders), batch, nmax,
                                               _ptr(green), _ptr(diag), _ptr(status),
                                               _stream_handle(stream)))
        return green, diag, status

    def profile(self, enable: bool) -> None:
        """Record CUDA events around every kernel of later evaluations."""
        L.check(self._lib.cdet_profile_enable(self._ctx, int(bool(enable))))

    def profile_read(self):
        """(per-stage milliseconds [split prep, assembly, minors, cdet],
        launches) since the last read; waits for the recorded events."""
        ms = (C.c_double * 4)(0.0, 0.0, 0.0, 0.0)
        launches = C.c_int64(0)
        L.check(self._lib.cdet_profile_read(self._ctx, ms, C.byref(launches)))
        return list(ms), launches.value

    def split_counters(self):
        """(accumulator columns written by the issued tcgen05.mma, each
        2 x 128 x 16 flops; coefficient-slice bytes streamed) of the last
        split-assembly evaluation; waits for it."""
        out = (C.c_uint64 * 2)(0, 0)
        L.check(self._lib.cdet_split_counters(self._ctx, out))
        return int(out[0]), int(out[1])

    # --------------------------------------------- reference entry points ---
    def evaluate_cdet_density_integrand_double(self, vertices) -> float:
        v = _as_vertex_array(vertices)
        order = v.shape[0]
        if order <= 0:
            raise RuntimeError("The replica integrand is defined only for order >= 1")
        values, status = self.integrand_batch(v[None], [order])
        if status[0] & L.CONFIG_BAD_INPUT:
            raise RuntimeError("Error (integrand): vertex coordinates rejected")
        if status[0] & L.CONFIG_NONFINITE:
            raise RuntimeError("Error (integrand): Value is not finite")
        return float(values[0])

    def evaluate_cdet_density_all_subset_integrands_double_into(self, vertices, values: List[float]) -> None:
        v = _as_vertex_array(vertices)
        env = v.shape[0]
        if env <= 1:
            raise RuntimeError("The all-subset replica integrand is defined only for envelope order >= 2")
        out, status = self.all_subsets_batch(v[None])
        if status[0] & L.CONFIG_BAD_INPUT:
            raise RuntimeError("Error (all-subset integrand): vertex coordinates rejected")
        if status[0] & L.CONFIG_NONFINITE:
            raise RuntimeError("Error (all-subset integrand): Value is not finite")
        values[:] = out[0].tolist()

    def evaluate_cdet_density_all_subset_integrands_double(self, vertices) -> List[float]:
        values: List[float] = []
        self.evaluate_cdet_density_all_subset_integrands_double_into(vertices, values)
        return values


def _stream_handle(stream) -> Optional[int]:
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


def subset_vertices(full_vertices, mask: int) -> np.ndarray:
    """subset_vertices (cdet_integrand_evaluator.h:592-602)."""
    v = _as_vertex_array(full_vertices)
    return v[[i for i in range(v.shape[0]) if (mask >> i) & 1]]
