// Device building blocks of the FP64 CDet integrand for sm_103a.
//
// Every floating-point operation on the FP64 path is written with an explicit
// round-to-nearest intrinsic (__dmul_rn, __dadd_rn, __dsub_rn, __fma_rn,
// __ddiv_rn). nvcc never contracts those, so each kernel performs the same
// IEEE operations, in the same order, as the reference integrand compiled for
// x86-64 (where no contraction happens and the explicit std::fma calls stay
// fused). On equal inputs the results are bit-identical to that build.
#pragma once

#include <cstdint>

namespace cdet {

constexpr int kWarp = 32;

// ------------------------------------------------------------- exact ops ---
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// ------------------------------------------------------- double-double ---
// Dekker/Knuth error-free transforms in the arrangement of the reference's
// DoubleDouble (utility/types.h:49-121).
struct DD {
    double hi, lo;
};

__device__ __forceinline__ double two_sum(double a, double b, double& err) {
    const double s = dadd(a, b);
    const double bb = dsub(s, a);
    err = dadd(dsub(a, dsub(s, bb)), dsub(b, bb));
    return s;
}
__device__ __forceinline__ double quick_two_sum(double a, double b, double& err) {
    const double s = dadd(a, b);
    err = dsub(b, dsub(s, a));
    return s;
}
__device__ __forceinline__ DD dd_add(DD x, DD y) {
    double s2, t2;
    double s1 = two_sum(x.hi, y.hi, s2);
    const double t1 = two_sum(x.lo, y.lo, t2);
    s2 = dadd(s2, t1);
    s1 = quick_two_sum(s1, s2, s2);
    s2 = dadd(s2, t2);
    DD r;
    r.hi = quick_two_sum(s1, s2, r.lo);
    return r;
}
__device__ __forceinline__ DD dd_sub(DD x, DD y) { return dd_add(x, DD{-y.hi, -y.lo}); }
__device__ __forceinline__ DD dd_mul(DD x, DD y) {
    const double p = dmul(x.hi, y.hi);
    double e = dfma(x.hi, y.hi, -p);
    e = dadd(e, dadd(dadd(dmul(x.hi, y.lo), dmul(x.lo, y.hi)), dmul(x.lo, y.lo)));
    DD r;
    r.hi = quick_two_sum(p, e, r.lo);
    return r;
}
__device__ __forceinline__ bool dd_finite(DD x) { return isfinite(x.hi) && isfinite(x.lo); }

// ------------------------------------------------------------ Clenshaw ---
// One row of a Chebyshev block: sum_{k<=degree} c[k] T_k(x) by the Clenshaw
// recurrence b_k = c_k + 2x b_{k+1} - b_{k+2} (g_funcs.h:395-418).
__device__ __forceinline__ double clenshaw_row(const double* __restrict__ c, int degree, double x) {
    if (degree < 0) return 0.0;
    if (degree == 0) return __ldg(c);
    if (degree == 1) return dadd(__ldg(c), dmul(__ldg(c + 1), x));
    const double two_x = dmul(2.0, x);
    double b1 = 0.0, b2 = 0.0;
#pragma unroll 8
    for (int k = degree; k >= 1; --k) {
        const double bk = dsub(dadd(__ldg(c + k), dmul(two_x, b1)), b2);
        b2 = b1;
        b1 = bk;
    }
    return dsub(dadd(__ldg(c), dmul(b1, x)), b2);
}

// Two blocks (spin up and down) evaluated together: the row recurrences run
// interleaved for instruction-level parallelism; the results equal two calls
// of clenshaw_row.
__device__ __forceinline__ void clenshaw_row_pair(const double* __restrict__ cu,
                                                  const double* __restrict__ cd, int degree,
                                                  double x, double& ru, double& rd) {
    if (degree < 2) {
        ru = clenshaw_row(cu, degree, x);
        rd = clenshaw_row(cd, degree, x);
        return;
    }
    const double two_x = dmul(2.0, x);
    double u1 = 0.0, u2 = 0.0, d1 = 0.0, d2 = 0.0;
#pragma unroll 4
    for (int k = degree; k >= 1; --k) {
        const double uk = dsub(dadd(__ldg(cu + k), dmul(two_x, u1)), u2);
        const double dk = dsub(dadd(__ldg(cd + k), dmul(two_x, d1)), d2);
        u2 = u1;
        u1 = uk;
        d2 = d1;
        d1 = dk;
    }
    ru = dsub(dadd(__ldg(cu), dmul(u1, x)), u2);
    rd = dsub(dadd(__ldg(cd), dmul(d1, x)), d2);
}

// Streaming form of the outer (u) Clenshaw sum over row values r_{nu-1}, ...,
// r_0 delivered in descending order. Feeding every row value exactly once
// gives the same operations as clenshaw_from_contiguous_coeffs over the full
// row array (g_funcs.h:742-747).
struct OuterClenshaw {
    double x, two_x, b1, b2, first, second;
    int degree;
    __device__ __forceinline__ void init(int deg, double xv) {
        degree = deg;
        x = xv;
        two_x = dmul(2.0, xv);
        b1 = b2 = 0.0;
        first = second = 0.0;
    }
    // Row value of index a (a runs from degree down to 0).
    __device__ __forceinline__ void push(int a, double r) {
        if (degree >= 2) {
            if (a >= 1) {
                const double bk = dsub(dadd(r, dmul(two_x, b1)), b2);
                b2 = b1;
                b1 = bk;
            } else {
                first = dsub(dadd(r, dmul(b1, x)), b2);
            }
        } else if (degree == 1) {
            if (a == 1) second = r;
            else first = dadd(r, dmul(second, x));
        } else {
            first = r;
        }
    }
    __device__ __forceinline__ double result() const { return first; }
};

// ------------------------------------------------- integer subset helpers ---
// Next integer with the same popcount (Gosper), for masks in increasing order.
__device__ __forceinline__ uint32_t next_same_popcount(uint32_t v) {
    const uint32_t t = v | (v - 1u);
    return (t + 1u) | (((~t & (t + 1u)) - 1u) >> (__ffs(v)));
}

// ------------------------------------------------- subsets by colex rank ---
// Binomial coefficients C(n, k) for n, k <= 24, built at compile time.
struct BinomialTable {
    uint32_t c[25][25];
};
constexpr BinomialTable make_binomial_table() {
    BinomialTable t{};
    for (int n = 0; n <= 24; ++n)
        for (int k = 0; k <= n; ++k) t.c[n][k] = (k == 0 || k == n) ? 1u : t.c[n - 1][k - 1] + t.c[n - 1][k];
    return t;
}
static __constant__ BinomialTable kBinomial = make_binomial_table();

// The m-subset of {0, ..., n-1} with colex rank r (r < C(n, m)), as a mask:
// its largest element is the largest c with C(c, m) <= r, and so on down.
// Work over the subsets of one size is spread evenly over lanes by rank.
__device__ __forceinline__ uint32_t colex_subset(uint32_t r, int m, int n) {
    uint32_t set = 0;
    int hi = n - 1;
    for (int i = m; i >= 1; --i) {
        int c = hi;
        while (c >= i && kBinomial.c[c][i] > r) --c;
        set |= 1u << c;
        r -= kBinomial.c[c][i];
        hi = c - 1;
    }
    return set;
}

}  // namespace cdet
