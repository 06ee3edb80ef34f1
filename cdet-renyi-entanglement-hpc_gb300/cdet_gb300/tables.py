"""Green-table precompute: piecewise 2-D Chebyshev tables of the free replica
Green functions, in the reference's table layout.

This is the table producer that feeds the integrand; it runs once per
parameter set, outside any timed region. It restates, batched over Chebyshev
nodes, the reference's

* square-lattice Hamiltonian (replica_free_greens.h:133-169),
* sector mixing matrices V^T diag(phase_m) V (:365-412),
* stable graded-replica kernel with diagonal scaling and a dense solve
  (stable_sector_kernel_eigenbasis, :414-496) and the eigen->site transform
  (:498-529),
* replica entries from the two sectors (replica_chebyshev_tables.h:489-510),
* Chebyshev node tables, the square->triangle node map and the per-sitepair
  2-D DCT (replica_chebyshev_tables.h:432-590),
* twisted and ordinary table builders (:592-695, :697-793).

The subsystem mask is an explicit site set, so the half-lattice masks of the
benchmark configurations (which the reference's named masks do not cover) are
built the same way as the named ones.

Table layout (the integrand's interface, replica_chebyshev_tables.h:25-38,
360-400): for each branch a float64 array of
``4 * S * S * nu * nv`` coefficients indexed
``(((((ra*2+rb)*N1 + x1)*N2 + y1)*N1 + x2)*N2 + y2) * nu*nv + a*nv + b``
and a corner array of ``4 * S * S`` values with the same site-pair index. The
ordinary table fills only its replica (0,0) quarter and indexes it by
``site1 * S + site2`` with ``site = y * N1 + x``, exactly as the reference
builder does (replica_chebyshev_tables.h:724-760); the lookup uses the
site-pair index above, which agrees with it on square lattices by the x<->y
symmetry of the ordinary Green function.

Arithmetic is float64 / complex128 via torch, on the CPU or on the GPU.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Dict, Optional, Sequence

import numpy as np
import torch

from .params import CdetParams


def square_lattice_hamiltonian(n1: int, n2: int, mu: float, t: float, pbc: bool) -> np.ndarray:
    """build_square_lattice_hamiltonian (replica_free_greens.h:133-169), with the
    same neighbour enumeration (so a periodic extent of 2 doubles the bond, as
    in the reference)."""
    s = n1 * n2
    h = np.zeros((s, s), dtype=np.float64)
    for y in range(n2):
        for x in range(n1):
            i = y * n1 + x
            h[i, i] = -mu
            neighbours = []
            if x + 1 < n1:
                neighbours.append((x + 1, y))
            elif pbc:
                neighbours.append((0, y))
            if y + 1 < n2:
                neighbours.append((x, y + 1))
            elif pbc:
                neighbours.append((x, 0))
            for xn, yn in neighbours:
                j = yn * n1 + xn
                h[i, j] -= t
                h[j, i] -= t
    return h


@dataclass
class NodeTables:
    node_u: np.ndarray  # (nu,) cos((2i+1) pi / (2 nu))
    node_v: np.ndarray
    dct_u: np.ndarray   # (nu, nu): alpha_a / nu * cos(a theta_i)
    dct_v: np.ndarray


def chebyshev_node_tables(nu: int, nv: int) -> NodeTables:
    """build_chebyshev_node_tables (replica_chebyshev_tables.h:432-471)."""
    def axis(n):
        theta = (2.0 * np.arange(n) + 1.0) * math.pi / (2.0 * n)
        nodes = np.cos(theta)
        a = np.arange(n)[:, None]
        alpha = np.where(a == 0, 1.0, 2.0)
        return nodes, alpha / n * np.cos(a * theta[None, :])
    nu_nodes, du = axis(nu)
    nv_nodes, dv = axis(nv)
    return NodeTables(nu_nodes, nv_nodes, du, dv)


def branch_node_times(tables: NodeTables, beta: float, upper: bool):
    """map_square_to_triangle (replica_chebyshev_tables.h:473-487) on every
    node, node index = i * nv + j. Returns (tau, tau_prime) arrays."""
    cu = np.repeat(tables.node_u, tables.node_v.size)
    cv = np.tile(tables.node_v, tables.node_u.size)
    if upper:
        tau = beta * (1.0 + cu) / 2.0
        tau_p = tau * (1.0 + cv) / 2.0
    else:
        tau_p = beta * (1.0 + cu) / 2.0
        tau = tau_p * (1.0 + cv) / 2.0
    return tau, tau_p


_LINALG_PRELOADED = False


def _preload_cuda_linalg() -> None:
    """Loads torch's CUDA linear-algebra library by its full path before the
    first batched solve on the GPU. torch opens it lazily by bare file name,
    which resolves through its own library's search path; a process whose
    dlopen calls are interposed (a profiler's launch capture) resolves the
    bare name without that path and fails. A library already loaded by its
    soname satisfies the later bare-name open."""
    global _LINALG_PRELOADED
    if _LINALG_PRELOADED:
        return
    _LINALG_PRELOADED = True
    import ctypes
    import os
    path = os.path.join(os.path.dirname(torch.__file__), "lib", "libtorch_cuda_linalg.so")
    if os.path.exists(path):
        ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)


class ReplicaGreenCalculator:
    """The free two-replica Green function of one spin species, in batches of
    imaginary-time nodes (ReplicaGreenCalculator, replica_free_greens.h:171-701)."""

    def __init__(self, n1: int, n2: int, beta: float, mu: float, pbc: bool,
                 mask_sites: Sequence[int], hopping_t: float = 1.0,
                 device: str = "cpu"):
        self.n1, self.n2, self.beta = n1, n2, float(beta)
        self.sites = n1 * n2
        self.device = torch.device(device)
        if self.device.type == "cuda":
            _preload_cuda_linalg()
        h = square_lattice_hamiltonian(n1, n2, float(mu), float(hopping_t), pbc)
        evals, evecs = np.linalg.eigh(h)
        self.eigenvalues = evals
        self.v = torch.tensor(evecs, dtype=torch.float64, device=self.device)
        in_mask = np.zeros(self.sites, dtype=bool)
        in_mask[list(mask_sites)] = True
        self.mixing = []
        for m in range(2):
            # omega_inverse_phase (replica_free_greens.h:668-677): -i (m=0) or
            # +i (m=1) inside subsystem A, 1 outside.
            phase = np.ones(self.sites, dtype=np.complex128)
            phase[in_mask] = -1j if m == 0 else 1j
            mix = evecs.T @ (phase[:, None] * evecs)
            self.mixing.append(torch.tensor(mix, dtype=torch.complex128, device=self.device))

    def sector_kernels(self, m: int, tau: np.ndarray, tau_p: np.ndarray, upper: bool) -> torch.Tensor:
        """Stable sector kernel in the eigenbasis for a batch of node times
        (stable_sector_kernel_eigenbasis, replica_free_greens.h:414-496)."""
        dev = self.device
        tf = torch.tensor(np.asarray(tau) / self.beta, dtype=torch.float64, device=dev)[:, None]
        tpf = torch.tensor(np.asarray(tau_p) / self.beta, dtype=torch.float64, device=dev)[:, None]
        theta = (tf + tpf) / 2.0 if upper else 1.0 - (tf + tpf) / 2.0
        x = torch.tensor(self.beta * self.eigenvalues, dtype=torch.float64, device=dev)[None, :]
        sx = x if upper else -x
        c = torch.clamp(sx, min=0.0)
        if upper:
            left_exp = (1.0 - tf) * x - (1.0 - theta) * c
            right_exp = tpf * x - theta * c
        else:
            left_exp = tf * sx - (1.0 - theta) * c
            right_exp = (1.0 - tpf) * sx - theta * c
        left = torch.exp(left_exp)
        rhs = torch.exp(right_exp)
        row_scale = torch.exp(-theta * c)
        col_scale = torch.exp(-(1.0 - theta) * c)
        diag = torch.exp(sx - c)
        mix = self.mixing[m] if upper else self.mixing[m].conj().transpose(0, 1)
        middle = row_scale[:, :, None].to(torch.complex128) * mix[None] * \
            col_scale[:, None, :].to(torch.complex128)
        idx = torch.arange(self.sites, device=dev)
        middle[:, idx, idx] += diag.to(torch.complex128).expand(middle.shape[0], -1)
        rhs_m = torch.diag_embed(rhs.to(torch.complex128))
        solved = torch.linalg.solve(middle, rhs_m)
        sign = 1.0 if upper else -1.0
        return (sign * left).to(torch.complex128)[:, :, None] * solved

    def green_sector(self, m: int, tau, tau_p, upper: bool) -> torch.Tensor:
        """Site-basis sector matrices G_m(tau, tau') = V K V^T (:498-529)."""
        k = self.sector_kernels(m, tau, tau_p, upper)
        v = self.v.to(torch.complex128)
        return v[None] @ k @ v.T[None]


def _replica_entries(g0: torch.Tensor, g1: torch.Tensor, n1: int, n2: int) -> torch.Tensor:
    """Replica entries for every site pair, in site-pair index order
    (replica_entry_from_sector_matrices, replica_chebyshev_tables.h:489-510).
    g0, g1: (K, S, S). Returns (K, 4*S*S) float64."""
    s = n1 * n2
    dev = g0.device
    # lookup position p = x*N2 + y  ->  site = y*N1 + x
    p = torch.arange(s, device=dev)
    site_of_p = (p % n2) * n1 + (p // n2)
    a = g0[:, site_of_p][:, :, site_of_p]
    b = g1[:, site_of_p][:, :, site_of_p]
    same = ((a + b) / 2.0).real
    diff = (a - b) / 2.0
    r01 = (1j * diff).real
    r10 = (-1j * diff).real
    k = g0.shape[0]
    return torch.stack([same, r01, r10, same], dim=1).reshape(k, 4 * s * s)


def _dct(samples: torch.Tensor, tables: NodeTables, nu: int, nv: int) -> torch.Tensor:
    """Per-sitepair 2-D DCT of a (nu*nv, F) sample grid into (F, nu*nv)
    Chebyshev coefficients (transform_sitepair_sample_grid_to_coeffs,
    replica_chebyshev_tables.h:552-590): C = Du S Dv^T."""
    dev = samples.device
    f = samples.shape[1]
    du = torch.tensor(tables.dct_u, dtype=torch.float64, device=dev)
    dv = torch.tensor(tables.dct_v, dtype=torch.float64, device=dev)
    grid = samples.reshape(nu, nv, f)
    t1 = torch.einsum("bj,ijf->ibf", dv, grid)
    coeffs = torch.einsum("ai,ibf->fab", du, t1)
    return coeffs.reshape(f, nu * nv)


def build_table(params: CdetParams, kind: str, device: str = "cpu",
                node_chunk: int = 2048) -> Dict[str, torch.Tensor]:
    """Build one resident table: kind in {"twisted_up", "twisted_down",
    "ordinary_up", "ordinary_down"} (load_data.h:35-47 with the per-kind
    mu - alpha_sigma and mask of chunked_load_data.h:582-609)."""
    twisted = kind.startswith("twisted")
    spin_up = kind.endswith("up")
    from .params import _dec
    mu = float(_dec(params.mu) - _dec(params.alpha_up if spin_up else params.alpha_down))
    mask = params.mask_sites if twisted else ()
    n1, n2, nu, nv = params.n1, params.n2, params.cheb_nu, params.cheb_nv
    s = n1 * n2
    beta = float(_dec(params.beta))
    calc = ReplicaGreenCalculator(n1, n2, beta, mu, params.pbc, mask,
                                  float(_dec(params.hopping_t)), device)
    nodes = chebyshev_node_tables(nu, nv)
    f_count = 4 * s * s
    out: Dict[str, torch.Tensor] = {}
    for upper in (True, False):
        key = "upper" if upper else "lower"
        g0c = calc.green_sector(0, np.zeros(1), np.zeros(1), upper)
        if twisted:
            g1c = calc.green_sector(1, np.zeros(1), np.zeros(1), upper)
            out[key + "_corners"] = _replica_entries(g0c, g1c, n1, n2)[0].contiguous()
        else:
            corners = torch.zeros(f_count, dtype=torch.float64, device=calc.device)
            corners[: s * s] = g0c[0].real.reshape(s * s)
            out[key + "_corners"] = corners
        tau, tau_p = branch_node_times(nodes, beta, upper)
        k_count = tau.size
        if twisted:
            samples = torch.empty((k_count, f_count), dtype=torch.float64, device=calc.device)
        else:
            samples = torch.empty((k_count, s * s), dtype=torch.float64, device=calc.device)
        for k0 in range(0, k_count, node_chunk):
            k1 = min(k_count, k0 + node_chunk)
            g0 = calc.green_sector(0, tau[k0:k1], tau_p[k0:k1], upper)
            if twisted:
                g1 = calc.green_sector(1, tau[k0:k1], tau_p[k0:k1], upper)
                samples[k0:k1] = _replica_entries(g0, g1, n1, n2)
            else:
                samples[k0:k1] = g0.real.reshape(k1 - k0, s * s)
            del g0
        coeffs = _dct(samples, nodes, nu, nv)
        del samples
        if twisted:
            out[key] = coeffs.reshape(-1).contiguous()
        else:
            full = torch.zeros((f_count, nu * nv), dtype=torch.float64, device=calc.device)
            full[: s * s] = coeffs
            out[key] = full.reshape(-1)
            del coeffs
    return out


def build_tables(params: CdetParams, device: str = "cpu") -> Dict[str, Dict[str, torch.Tensor]]:
    """All four resident tables. When ALPHA_UP == ALPHA_DOWN the down tables
    are the up tables (load_data.h:70-91), shared here without a copy."""
    tables = {"twisted_up": build_table(params, "twisted_up", device),
              "ordinary_up": build_table(params, "ordinary_up", device)}
    if params.alpha_equal:
        tables["twisted_down"] = tables["twisted_up"]
        tables["ordinary_down"] = tables["ordinary_up"]
    else:
        tables["twisted_down"] = build_table(params, "twisted_down", device)
        tables["ordinary_down"] = build_table(params, "ordinary_down", device)
    return tables


def table_bytes(params: CdetParams) -> int:
    """Bytes of one branch of one table in the reference layout."""
    s = params.sites
    return 4 * s * s * params.cheb_nu * params.cheb_nv * 8
