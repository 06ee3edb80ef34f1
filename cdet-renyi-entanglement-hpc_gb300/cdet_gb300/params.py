"""Parameter set of the CDet integrand and its runtime scalars.

Mirrors the process globals the reference integrand reads
(include/cdet/parameters.h:11-33, precision_config.h:208-287) and the scalars
it derives from them once per parameter set
(make_integrand_runtime_scalars, integrand_replica_randomly_sampled.h:98-119).

The reference derives the scalars in double-double / 100-digit arithmetic from
decimal parameter strings and rounds each to double. Here the same quantities
are computed with 60-digit decimal arithmetic and rounded to double, which
gives the same doubles (the scalars are correctly rounded in both).
"""
from __future__ import annotations

import dataclasses
import decimal
from typing import Sequence, Tuple

_CTX = decimal.Context(prec=60)


def _dec(value) -> decimal.Decimal:
    return _CTX.create_decimal(str(value))


@dataclasses.dataclass(frozen=True)
class CdetParams:
    """One parameter set, with the reference's params.txt key in each comment.

    Lattice sites are indexed ``site = y * n1 + x`` (replica_free_greens.h:28-33).
    ``mask_sites`` is the replica-swap subsystem A as a tuple of site indices;
    the helpers below build the reference's named masks and the half-lattice
    mask the benchmark configurations use.
    """

    n1: int                       # N1
    n2: int                       # N2
    beta: str = "2.0"             # BETA
    mu: str = "0.0"               # MU
    u: str = "2.0"                # U
    alpha_up: str = "0.0"         # ALPHA_UP
    alpha_down: str = "0.0"       # ALPHA_DOWN
    pbc: bool = True              # PBC
    mask_sites: Tuple[int, ...] = ()  # SUBREGION_MASK (as explicit sites)
    cheb_nu: int = 12             # CHEB_NU
    cheb_nv: int = 12             # CHEB_NV
    branch_epsilon: str = "1e-13"  # BRANCH_EPSILON
    tol_fpm: str = "1e-7"         # TOL_FPM
    fpm_global_shift: str = "auto"  # FPM_GLOBAL_SHIFT ("auto" -> -1)
    z_epsilon0: str = "auto"      # ZTRANSFORM_EPSILON0 ("auto" -> 2e-16 in double)
    z_safety: str = "1e4"         # ZTRANSFORM_SAFETY_FACTOR
    hopping_t: str = "1.0"        # t (fixed to 1 in the reference, replica_free_greens.h:188)

    @property
    def sites(self) -> int:
        return self.n1 * self.n2

    @property
    def alpha_equal(self) -> bool:
        """True when ALPHA_UP == ALPHA_DOWN: the reference then builds one table
        per set and uses it for both spins (load_data.h:70-91)."""
        return _dec(self.alpha_up) == _dec(self.alpha_down)

    def runtime_scalars(self) -> dict:
        """The doubles the integrand uses (IntegrandRuntimeScalars<double>)."""
        beta = _dec(self.beta)
        u = _dec(self.u)
        if u == 0:
            raise ValueError("U must be non-zero: the diagonal shifts are alpha / U")
        scale = _CTX.sqrt(u * self.n1 * self.n2 * beta)
        shift = (-1.0 if self.fpm_global_shift.strip().lower() == "auto"
                 else float(_dec(self.fpm_global_shift)))
        eps0 = (2.0e-16 if self.z_epsilon0.strip().lower() == "auto"
                else float(_dec(self.z_epsilon0)))
        return {
            "n1": self.n1,
            "n2": self.n2,
            "cheb_nu": self.cheb_nu,
            "cheb_nv": self.cheb_nv,
            "beta": float(beta),
            "u": float(u),
            "branch_eps": float(_dec(self.branch_epsilon)),
            "scale": float(scale),
            "diag_up_shift": float(_CTX.divide(_dec(self.alpha_down), u)),
            "diag_down_shift": float(_CTX.divide(_dec(self.alpha_up), u)),
            "tol_fpm": float(_dec(self.tol_fpm)),
            "fpm_shift": shift,
            "z_eps0": eps0,
            "z_safety": float(_dec(self.z_safety)),
        }


def dd_of_literal(literal, significand_bits: int = 0) -> Tuple[float, float]:
    """DoubleDouble(MP_Real(literal)) (utility/types.h:41-45): the nearest
    double to the value, then the nearest double to the rest. The reference's
    MP_Real holds 100 decimal digits, so the value is the literal itself
    (significand_bits = 0); significand_bits = 113 first rounds it to IEEE
    binary128, as a build whose MP_Real is quad precision does."""
    from fractions import Fraction
    x = Fraction(_dec(literal))
    if significand_bits and x != 0:
        sign = -1 if x < 0 else 1
        a = abs(x)
        e = a.numerator.bit_length() - a.denominator.bit_length()  # 2^e <= a < 2^(e+2)
        if Fraction(2) ** e > a:
            e -= 1
        scale = Fraction(2) ** (significand_bits - 1 - e)
        n = a * scale
        q, r = divmod(n.numerator, n.denominator)
        twice = 2 * r
        if twice > n.denominator or (twice == n.denominator and q % 2 == 1):
            q += 1
        x = sign * Fraction(q) / scale
    hi = float(x)
    lo = float(x - Fraction(hi))
    return hi, lo


def dd_scalars(params: "CdetParams", significand_bits: int = 0) -> dict:
    """The DoubleDouble values the reference's INTEGRAND_REAL=double_double
    mode reads (cdet_dd_scalars): beta, U, the alphas, TOL_FPM,
    FPM_GLOBAL_SHIFT (-1 when auto), ZTRANSFORM_EPSILON0 (1e-31 when auto,
    precision_config.h:173-186) and ZTRANSFORM_SAFETY_FACTOR."""
    def lit(v: str, auto: str) -> str:
        return auto if v.strip().lower() == "auto" else v
    return {
        "beta": dd_of_literal(params.beta, significand_bits),
        "u": dd_of_literal(params.u, significand_bits),
        "alpha_up": dd_of_literal(params.alpha_up, significand_bits),
        "alpha_down": dd_of_literal(params.alpha_down, significand_bits),
        "tol_fpm": dd_of_literal(params.tol_fpm, significand_bits),
        "fpm_shift": dd_of_literal(lit(params.fpm_global_shift, "-1"), significand_bits),
        "z_eps0": dd_of_literal(lit(params.z_epsilon0, "1e-31"), significand_bits),
        "z_safety": dd_of_literal(params.z_safety, significand_bits),
    }


def site_index(x: int, y: int, n1: int) -> int:
    return y * n1 + x


def named_mask(name: str, n1: int, n2: int, radius: int = 0) -> Tuple[int, ...]:
    """The reference's named subsystem masks (replica_free_greens.h:20-131)."""
    key = name.strip().lower().replace("-", "_")
    out = []
    for y in range(n2):
        for x in range(n1):
            if key in ("empty", "none", "ordinary"):
                inside = False
            elif key == "checkerboard":
                inside = (x + y) % 2 == 0
            elif key == "first_row":
                inside = y == 0
            elif key == "first_column":
                inside = x == 0
            elif key in ("origin_square", "center_square", "centered_square"):
                inside = _in_origin_square(x, n1, radius) and _in_origin_square(y, n2, radius)
            else:
                raise ValueError(f"unknown subregion mask {name!r}")
            if inside:
                out.append(site_index(x, y, n1))
    return tuple(sorted(out))


def _in_origin_square(c: int, extent: int, radius: int) -> bool:
    if radius <= 0:
        return False
    if 2 * radius >= extent:
        return True
    return c < radius or c >= extent - radius


def half_lattice_mask(n1: int, n2: int) -> Tuple[int, ...]:
    """Subsystem A = the x < n1/2 half of the lattice (an (n1/2) x n2 strip).

    The reference has no such named mask; the table precompute here accepts
    any explicit site set, so the half-lattice configurations use this one.
    """
    return tuple(sorted(site_index(x, y, n1) for y in range(n2) for x in range(n1 // 2)))


def with_sites(params: CdetParams, sites: Sequence[int]) -> CdetParams:
    return dataclasses.replace(params, mask_sites=tuple(sorted(int(s) for s in sites)))
