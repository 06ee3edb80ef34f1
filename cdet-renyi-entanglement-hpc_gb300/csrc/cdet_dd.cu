// The reference's double-double integrand mode on the GPU:
// INTEGRAND_REAL=double_double with VECTOR_REAL=double
// (cdet_integrand_evaluator.h:431-465, precision_config.h:15-26).
//
// The Green matrices are the FP64 form's (the same Clenshaw sums, shifts and
// scale in double, integrand_replica_randomly_sampled.h:434-484). Each entry
// is widened to DoubleDouble(x, 0), and from there every operation is the
// reference's DoubleDouble arithmetic (utility/types.h:30-182) in the
// reference's order: the shifted Schur-complement recursion with its
// whole-matrix LU fallback (fast_principle_minors.h:39-246), the connected
// recursion with the round-off filter (integrand_replica_randomly_sampled.h:
// 226-290), the double-double prefactor and twisted - 2 ordinary. The order-1
// branch widens the unshifted diagonal value and adds the DoubleDouble shifts
// alpha / U (:173-213). With the reference's DoubleDouble being error-free
// transforms of doubles, the values are the reference's bit for bit.
//
// One persistent kernel after the assembly: warps take configurations from
// the order-sorted slots (decreasing order) through an atomic queue head; a
// warp runs one configuration's minors and recursion in its shared-memory
// workspace (the compact minors layout in DoubleDouble elements, A and one
// arena per spin: 40.5 KB per warp at order 10 with one spin per set, five
// warps per SM), the masks of a popcount level dealt to its lanes, each mask's
// submask sum on one lane in the reference's order.
#include "cdet_device.cuh"
#include "cdet_kernels.cuh"

#include <algorithm>

namespace cdet {

namespace {

// ------------------------------------------------ DoubleDouble (the rest) ---
// operator/ (utility/types.h:114-120): q1 = x.hi / y.hi, the remainder
// x - q1 y, q2 = (r.hi + r.lo) / y.hi, q1 + q2 renormalised.
__device__ __forceinline__ DD dd_div(DD x, DD y) {
    const double q1 = ddiv(x.hi, y.hi);
    const DD r = dd_sub(x, dd_mul(DD{q1, 0.0}, y));
    const double q2 = ddiv(dadd(r.hi, r.lo), y.hi);
    DD q = dd_add(DD{q1, 0.0}, DD{q2, 0.0});
    const double s = dadd(q.hi, q.lo);
    q.lo = dsub(q.lo, dsub(s, q.hi));
    q.hi = s;
    return q;
}
// dd_abs (utility/types.h:221-223)
__device__ __forceinline__ DD dd_abs(DD x) { return x.hi < 0.0 ? DD{-x.hi, -x.lo} : x; }
// the comparison operators (utility/types.h:146-168): lexicographic on (hi, lo)
__device__ __forceinline__ bool dd_lt(DD a, DD b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool dd_gt(DD a, DD b) { return dd_lt(b, a); }
__device__ __forceinline__ bool dd_eq(DD a, DD b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool dd_zero(DD a) { return a.hi == 0.0 && a.lo == 0.0; }
// subtract_product for DoubleDouble (fast_principle_minors.h:30-37): base - left * right
__device__ __forceinline__ DD dd_sub_prod(DD left, DD right, DD base) { return dd_sub(base, dd_mul(left, right)); }

// The lighter steps used on the split assembly's Green matrices, where the
// reference's values are not the contract: products as FMAs without the
// lo x lo term, sums as one two-sum of the highs plus the lows and one
// renormalisation (relative error a few 2^-104 of the operands).
__device__ __forceinline__ DD dd_mul_light(DD x, DD y) {
    const double p = dmul(x.hi, y.hi);
    double e = dfma(x.hi, y.hi, -p);
    e = dfma(x.hi, y.lo, e);
    e = dfma(x.lo, y.hi, e);
    DD r;
    r.hi = quick_two_sum(p, e, r.lo);
    return r;
}
__device__ __forceinline__ DD dd_add_light(DD x, DD y) {
    double e;
    const double s = two_sum(x.hi, y.hi, e);
    e = dadd(e, dadd(x.lo, y.lo));
    DD r;
    r.hi = quick_two_sum(s, e, r.lo);
    return r;
}
// base - left * right with the product as FMAs
__device__ __forceinline__ DD dd_sub_prod_light(DD left, DD right, DD base) {
    const double p = dmul(left.hi, right.hi);
    double pe = dfma(left.hi, right.hi, -p);
    pe = dfma(left.hi, right.lo, pe);
    pe = dfma(left.lo, right.hi, pe);
    double e;
    const double s = two_sum(base.hi, -p, e);
    e = dadd(e, dsub(base.lo, pe));
    DD r;
    r.hi = quick_two_sum(s, e, r.lo);
    return r;
}
template <bool Exact>
__device__ __forceinline__ DD mul_t(DD x, DD y) { return Exact ? dd_mul(x, y) : dd_mul_light(x, y); }
template <bool Exact>
__device__ __forceinline__ DD add_t(DD x, DD y) { return Exact ? dd_add(x, y) : dd_add_light(x, y); }
template <bool Exact>
__device__ __forceinline__ DD sub_prod_t(DD l, DD r, DD b) {
    return Exact ? dd_sub_prod(l, r, b) : dd_sub_prod_light(l, r, b);
}

__device__ __forceinline__ DD shfl_dd(DD v, int src_lane_xor) {
    return DD{__shfl_xor_sync(0xffffffffu, v.hi, src_lane_xor), __shfl_xor_sync(0xffffffffu, v.lo, src_lane_xor)};
}

// determinant_principal_minor_from_buffer<DoubleDouble> (fast_principle_minors.h:39-105)
// for one mask on one lane; m is this lane's n x n DoubleDouble scratch.
__device__ DD minor_by_lu_dd(const DD* a, int n, uint32_t mask, DD* m) {
    int idx[kMaxOrder];
    int k = 0;
    for (int i = 0; i < n; ++i)
        if (mask & (1u << i)) idx[k++] = i;
    if (k == 0) return DD{1.0, 0.0};
    for (int r = 0; r < k; ++r)
        for (int c = 0; c < k; ++c) m[r * k + c] = a[idx[r] * n + idx[c]];
    DD det{1.0, 0.0};
    int sign = 1;
    for (int col = 0; col < k; ++col) {
        int pivot_row = col;
        DD pivot_abs = dd_abs(m[col * k + col]);
        for (int row = col + 1; row < k; ++row) {
            const DD cand = dd_abs(m[row * k + col]);
            if (dd_gt(cand, pivot_abs)) {
                pivot_abs = cand;
                pivot_row = row;
            }
        }
        if (dd_zero(pivot_abs)) return DD{0.0, 0.0};
        if (pivot_row != col) {
            for (int c = col; c < k; ++c) {
                const DD t = m[col * k + c];
                m[col * k + c] = m[pivot_row * k + c];
                m[pivot_row * k + c] = t;
            }
            sign = -sign;
        }
        const DD pivot = m[col * k + col];
        det = dd_mul(det, pivot);
        for (int row = col + 1; row < k; ++row) {
            const DD factor = dd_div(m[row * k + col], pivot);
            if (dd_zero(factor)) continue;
            m[row * k + col] = DD{0.0, 0.0};
            for (int c = col + 1; c < k; ++c) m[row * k + c] = dd_sub_prod(factor, m[col * k + c], m[row * k + c]);
        }
    }
    return sign < 0 ? DD{-det.hi, -det.lo} : det;
}

// mat2pm_from_buffer<DoubleDouble> (fast_principle_minors.h:120-246) for one
// matrix on one warp: shifted[mask] (mask >= 1) ends as the principal minor of
// the rows and columns in mask. Returns true when the LU fallback ran.
// Exact: the reference's operations; otherwise the lighter steps for the
// Schur updates, the minor sums and products and the shift removal (the
// pivots, their inverses and the fallback decision stay exact).
template <bool Exact>
__device__ bool mat2pm_dd_warp(const DD* A, int n, DD tol, DD thresh, const WsLayout& lay, DD* ws, DD* shifted,
                               DD* lu_lane, int lane) {
    const int msize = n * n;
    const uint32_t subsets = 1u << n;
    const DD zero{0.0, 0.0};
    DD max_abs = zero;  // the first maximal entry, as the sequential scan keeps it
    for (int k = lane; k < msize; k += kWarp) {
        const DD e = dd_abs(A[k]);
        if (dd_gt(e, max_abs)) max_abs = e;
    }
    for (int off = 16; off > 0; off >>= 1) {
        const DD o = shfl_dd(max_abs, off);
        if (dd_gt(o, max_abs)) max_abs = o;
    }
    const bool explicit_shift = !dd_lt(thresh, zero);
    const DD p = explicit_shift ? thresh : dd_div(max_abs, DD{static_cast<double>(msize), 0.0});
    if (dd_eq(max_abs, zero) && dd_eq(p, zero)) {
        for (uint32_t m = lane; m < subsets; m += kWarp) shifted[m] = zero;
        __syncwarp();
        return false;
    }
    const DD fallback_eps = (dd_gt(tol, zero) && dd_gt(max_abs, zero)) ? dd_mul(tol, max_abs) : zero;
    const bool eps_on = dd_gt(fallback_eps, zero);
    // The compact arena (compact_minors_layout): the level lists share
    // shifted's arena with the minors, each node's pivot inverse replaces its
    // pivot entry and its factors column 0, each shifted minor is written once
    // as p + its pivot entry (the initialise-then-add form's value).
    DD* old_list = shifted + compact_list_offset(n, 0, lay.arena);
    DD* new_list = nullptr;
    for (int k = lane; k < msize; k += kWarp) old_list[k] = A[k];
    if (lane == 0) shifted[0] = DD{1.0, 0.0};
    __syncwarp();
    if (lane == 0) shifted[1] = dd_add(p, old_list[0]);
    __syncwarp();
    uint32_t minor_index = 2;
    bool fell_back = false;
    for (int level = 0; level < n - 1; ++level) {
        const int old_size = n - level;
        const int old_msize = old_size * old_size;
        const int new_size = old_size - 1;
        const int new_msize = new_size * new_size;
        const int sets = 1 << level;
        bool bad_pivot = false;
        for (int set = lane; set < sets; set += kWarp) {
            const DD pivot = dd_add(old_list[set * old_msize], p);
            const DD pa = dd_abs(pivot);
            if (dd_eq(pa, zero) || (eps_on && !dd_gt(pa, fallback_eps))) bad_pivot = true;
            old_list[set * old_msize] = dd_div(DD{1.0, 0.0}, pivot);
        }
        if (__any_sync(0xffffffffu, bad_pivot)) {
            fell_back = true;
            break;
        }
        __syncwarp();
        for (int item = lane; item < sets * new_size; item += kWarp) {
            const int set = item / new_size;
            const int row = item - set * new_size;
            DD* entry = old_list + set * old_msize + (row + 1) * old_size;
            *entry = mul_t<Exact>(*entry, old_list[set * old_msize]);
        }
        __syncwarp();
        if (level == n - 2) {
            // the last level's 1 x 1 children, straight to their shifted minors
            for (int set = lane; set < sets; set += kWarp) {
                const DD* m = old_list + set * 4;
                const DD base = m[3];
                shifted[minor_index + set] = add_t<Exact>(p, base);
                shifted[minor_index + sets + set] = add_t<Exact>(p, sub_prod_t<Exact>(m[1], m[2], base));
            }
            __syncwarp();
            minor_index += 2 * sets;
            break;
        }
        new_list = shifted + compact_list_offset(n, level + 1, lay.arena);
        const int items = sets * new_msize;
#pragma unroll 4
        for (int item = lane; item < items; item += kWarp) {  // independent items: chains in flight
            const int set = item / new_msize;
            const int e = item - set * new_msize;
            const int row = e / new_size;
            const int col = e - row * new_size;
            const int src = set * old_msize;
            const DD base = old_list[src + (row + 1) * old_size + col + 1];
            new_list[item] = base;
            new_list[items + item] =
                sub_prod_t<Exact>(old_list[src + 1 + col], old_list[src + (row + 1) * old_size], base);
        }
        __syncwarp();
        for (int m = lane; m < 2 * sets; m += kWarp)
            shifted[minor_index + m] = add_t<Exact>(p, new_list[m * new_msize]);
        minor_index += 2 * sets;
        old_list = new_list;
        __syncwarp();
    }
    if (fell_back) {
        // determinant_principal_minors_from_buffer<DoubleDouble> (fast_principle_minors.h:107-115)
        for (uint32_t m = 1 + lane; m < subsets; m += kWarp) shifted[m] = minor_by_lu_dd(A, n, m, lu_lane);
        __syncwarp();
        return true;
    }
    for (uint32_t step = 1; step < subsets; step <<= 1) {  // the prefix product over levels
#pragma unroll 4
        for (uint32_t set = step + 1 + lane; set < 2 * step; set += kWarp)
            shifted[set] = mul_t<Exact>(shifted[set], shifted[set - step]);
        __syncwarp();
    }
    for (uint32_t step = subsets; step > 1; step >>= 1) {  // the shift removal, bit by bit from the top
        const uint32_t half = step >> 1;
        const int hb = __ffs(half) - 1;  // half = 2^hb
#pragma unroll 4
        for (uint32_t q = lane; q < subsets / 2; q += kWarp) {
            const uint32_t ss = ((q >> hb) << (hb + 1)) + half + (q & (half - 1u));
            shifted[ss] = sub_prod_t<Exact>(p, shifted[ss - half], shifted[ss]);
        }
        __syncwarp();
    }
    return false;
}

// compute_dp_ztransform<DoubleDouble> (integrand_replica_randomly_sampled.h:
// 226-290) on one warp for order n >= 2: a[mask] for every mask, dp of the
// masks holding vertex 0 into dp_s[mask >> 1]; each mask's submask sum on one
// lane, its terms in the reference's descending order.
__device__ DD cdet_dd_warp(const DD* a, DD* dp_s, int n, DD threshold, int lane) {
    const DD zero{0.0, 0.0};
    const bool filter = dd_gt(threshold, zero);
    if (lane == 0) dp_s[0] = a[1];
    __syncwarp();
    const int nbits = n - 1;
    for (int k = 2; k <= n; ++k) {
        const int kk = k - 1;
        const uint32_t masks = kBinomial.c[nbits][kk];
        for (uint32_t idx = lane; idx < masks; idx += kWarp) {
            const uint32_t rest = colex_subset(idx, kk, nbits);
            DD acc = a[(rest << 1) | 1u];
            DD rhs = dd_abs(acc);
            for (uint32_t sm = (rest - 1u) & rest;; sm = (sm - 1u) & rest) {
                const DD term = dd_mul(dp_s[sm], a[(rest ^ sm) << 1]);
                acc = dd_sub(acc, term);
                rhs = dd_add(rhs, dd_abs(term));
                if (sm == 0) break;
            }
            if (filter && dd_lt(dd_abs(acc), dd_mul(threshold, rhs))) acc = zero;
            dp_s[rest] = acc;
        }
        __syncwarp();  // the next level reads this one
    }
    return dp_s[(1u << nbits) - 1u];
}

// One set of configuration c (order n): its prefactored DoubleDouble value.
__device__ DD dd_set_value(const Problem& p, const Scratch& w, int64_t c, int set, int n, const WsLayout& lay,
                           DD* ws, DD* lu_lane, int lane, int32_t& status) {
    const int nmax = p.max_order;
    const int r = set == 0 ? 2 : 1;
    if (n == 1) {
        // order1_density_integrand_from_sampled_vertex (:173-213) with
        // IntegrandRealT = DoubleDouble: the unshifted diagonal widened, the
        // DoubleDouble shifts added; no finiteness check on this branch
        const double* diag = w.diag + c * 2 * 2 * nmax;
        const DD su = dd_add(DD{diag[(set * 2) * nmax], 0.0}, DD{p.dd_shift[0].hi, p.dd_shift[0].lo});
        const DD sd = dd_add(DD{diag[(set * 2 + 1) * nmax], 0.0}, DD{p.dd_shift[1].hi, p.dd_shift[1].lo});
        const DD counter = dd_mul(DD{p.dd_shift[0].hi, p.dd_shift[0].lo}, DD{p.dd_shift[1].hi, p.dd_shift[1].lo});
        const DD ru = dd_mul(dd_mul(DD{static_cast<double>(-r), 0.0}, DD{p.dd_u.hi, p.dd_u.lo}),
                             DD{p.dd_beta.hi, p.dd_beta.lo});
        return dd_mul(ru, dd_sub(dd_mul(su, sd), counter));
    }
    const double* green = w.green + (c * 2 + set) * 2 * static_cast<int64_t>(nmax) * nmax;
    DD* A = ws + lay.a;
    const DD tol{p.dd_tol.hi, p.dd_tol.lo}, thresh{p.dd_fpm_shift.hi, p.dd_fpm_shift.lo};
    bool fb = false;
    for (int k = lane; k < n * n; k += kWarp) A[k] = DD{green[k], 0.0};
    __syncwarp();
    DD* su = ws + lay.shifted_up;
    fb |= mat2pm_dd_warp<true>(A, n, tol, thresh, lay, ws, su, lu_lane, lane);
    const bool one_spin = p.same_spin[set] != 0;
    if (!one_spin) {
        for (int k = lane; k < n * n; k += kWarp) A[k] = DD{green[static_cast<int64_t>(nmax) * nmax + k], 0.0};
        __syncwarp();
        fb |= mat2pm_dd_warp<true>(A, n, tol, thresh, lay, ws, ws + lay.shifted_down, lu_lane, lane);
    }
    const DD* sd = one_spin ? su : ws + lay.shifted_down;
    // a[mask] = up[mask - 1] * down[mask - 1] (:254-257), in place of the up minors
    for (uint32_t m = lane; m < (1u << n); m += kWarp) su[m] = m == 0 ? DD{0.0, 0.0} : dd_mul(su[m], sd[m]);
    __syncwarp();
    const DD top = cdet_dd_warp(su, ws + lay.old_list, n, DD{p.dd_threshold.hi, p.dd_threshold.lo}, lane);
    const DD value = dd_mul(DD{p.pref_dd[set][n].hi, p.pref_dd[set][n].lo}, top);
    if (!dd_finite(value)) status |= kStatusNonFinite;
    if (fb) status |= kStatusFpmFallback;
    __syncwarp();  // the next set reuses the workspace
    return value;
}

__global__ void __launch_bounds__(kDDMaxWarps * 32) integrand_dd(const __grid_constant__ Problem p,
                                                   const __grid_constant__ Scratch w) {
    extern __shared__ double dd_smem[];
    const int lane = threadIdx.x & (kWarp - 1);
    const int warp_in_block = threadIdx.x / kWarp;
    const int warps_per_block = blockDim.x / kWarp;
    const int64_t global_warp = static_cast<int64_t>(blockIdx.x) * warps_per_block + warp_in_block;
    const int nmax = p.max_order;
    const WsLayout lay = compact_minors_layout(nmax, !(p.same_spin[0] && p.same_spin[1]), true);
    DD* ws = reinterpret_cast<DD*>(dd_smem) + static_cast<size_t>(warp_in_block) * lay.total;
    // a lane's LU-fallback matrix: two lanes' FP64 regions of the scratch
    DD* lu_lane = reinterpret_cast<DD*>(w.lu_scratch + (static_cast<size_t>(global_warp) * kWarp + lane) * 2 *
                                                           nmax * nmax);
    uint32_t* head = w.order_count + kQueueHeadIndex;
    const uint32_t batch = static_cast<uint32_t>(p.batch);
    for (;;) {
        uint32_t slot = 0;
        if (lane == 0) slot = atomicAdd(head, 1u);
        slot = __shfl_sync(0xffffffffu, slot, 0);
        if (slot >= batch) break;
        const int64_t c = __ldg(w.config_at + slot);
        const int n = __ldg(p.orders + c);
        if (n < 1 || n > nmax) continue;  // flagged by the assembly
        int32_t status = 0;
        const DD twisted = dd_set_value(p, w, c, 0, n, lay, ws, lu_lane, lane, status);
        const DD ordinary = dd_set_value(p, w, c, 1, n, lay, ws, lu_lane, lane, status);
        if (lane == 0) {
            // twisted - DoubleDouble(2) * ordinary (cdet_integrand_evaluator.h:233-263), then to double
            const DD result = dd_sub(twisted, dd_mul(DD{2.0, 0.0}, ordinary));
            p.values[c] = dadd(result.hi, result.lo);
            if (status) atomicOr(p.status + c, status);
        }
    }
}

// ---- lane form: minors by warps into lane-interleaved a, CDet by lanes ----
// For large batches: principal_minors_dd gives each (configuration, set) a
// warp, as the FP64 form does, and writes a = up * down into [group][set]
// [mask][lane] (the slot's lane of its order-sorted group of 32); cdet_dd_lane
// then gives each slot a lane, so the 32 lanes of a warp run the recursions of
// 32 configurations of (nearly) one order in step, every load a coalesced
// 512-byte row. The same operations as the warp form: the same values.
__device__ __forceinline__ DD* lane_a(const Scratch& w, int64_t slot, int set, int nmax) {
    const int64_t subsets = int64_t{1} << nmax;
    return reinterpret_cast<DD*>(w.dd_lanes) + ((slot >> 5) * 2 + set) * subsets * kWarp + (slot & 31);
}
__device__ __forceinline__ DD* lane_dp(const Scratch& w, int64_t slot, int set, int nmax, int64_t groups) {
    const int64_t subsets = int64_t{1} << nmax;
    return reinterpret_cast<DD*>(w.dd_lanes) + groups * 2 * subsets * kWarp +
           ((slot >> 5) * 2 + set) * (subsets / 2) * kWarp + (slot & 31);
}

template <bool Exact>
__global__ void __launch_bounds__(kDDMaxWarps * 32) principal_minors_dd(const __grid_constant__ Problem p,
                                                          const __grid_constant__ Scratch w) {
    extern __shared__ double dd_smem[];
    const int lane = threadIdx.x & (kWarp - 1);
    const int warp_in_block = threadIdx.x / kWarp;
    const int warps_per_block = blockDim.x / kWarp;
    const int64_t global_warp = static_cast<int64_t>(blockIdx.x) * warps_per_block + warp_in_block;
    const int64_t total_warps = static_cast<int64_t>(gridDim.x) * warps_per_block;
    const int nmax = p.max_order;
    const WsLayout lay = compact_minors_layout(nmax, !(p.same_spin[0] && p.same_spin[1]), true);
    DD* ws = reinterpret_cast<DD*>(dd_smem) + static_cast<size_t>(warp_in_block) * lay.total;
    DD* lu_lane = reinterpret_cast<DD*>(w.lu_scratch + (static_cast<size_t>(global_warp) * kWarp + lane) * 2 *
                                                           nmax * nmax);
    const DD tol{p.dd_tol.hi, p.dd_tol.lo}, thresh{p.dd_fpm_shift.hi, p.dd_fpm_shift.lo};
    for (int64_t item = global_warp; item < p.batch * 2; item += total_warps) {
        const int64_t c = item >> 1;
        const int set = static_cast<int>(item & 1);
        const int n = __ldg(p.orders + c);
        if (n < 2 || n > nmax) continue;  // order 1 needs no minors
        const double* green = w.green + (c * 2 + set) * 2 * static_cast<int64_t>(nmax) * nmax;
        DD* A = ws + lay.a;
        bool fb = false;
        for (int k = lane; k < n * n; k += kWarp) A[k] = DD{green[k], 0.0};
        __syncwarp();
        DD* su = ws + lay.shifted_up;
        fb |= mat2pm_dd_warp<Exact>(A, n, tol, thresh, lay, ws, su, lu_lane, lane);
        const bool one_spin = p.same_spin[set] != 0;
        if (!one_spin) {
            for (int k = lane; k < n * n; k += kWarp) A[k] = DD{green[static_cast<int64_t>(nmax) * nmax + k], 0.0};
            __syncwarp();
            fb |= mat2pm_dd_warp<Exact>(A, n, tol, thresh, lay, ws, ws + lay.shifted_down, lu_lane, lane);
        }
        const DD* sd = one_spin ? su : ws + lay.shifted_down;
        DD* a = lane_a(w, __ldg(w.slot_of + c), set, nmax);
        for (uint32_t m = lane; m < (1u << n); m += kWarp)
            a[static_cast<int64_t>(m) * kWarp] = m == 0 ? DD{0.0, 0.0} : mul_t<Exact>(su[m], sd[m]);
        if (fb && lane == 0) atomicOr(p.status + c, kStatusFpmFallback);
        __syncwarp();
    }
}

// compute_dp_ztransform<DoubleDouble> for the slot's configuration on one
// lane, masks holding vertex 0 in popcount order, each one's submasks in the
// reference's descending order; then the prefactors and the combine.
// Exact: the reference's DoubleDouble operations (51 FP64 operations per
// pair update). Otherwise (the split assembly's Green matrices, where the
// reference's values are not the contract): the product as FMAs without the
// lo x lo term, the subtraction as one two-sum of the highs plus the lows and
// one renormalisation, and the round-off filter's magnitude sum in FP64 on
// the products' high parts (16 operations; the accumulated error stays near
// 1e-32 of the terms' magnitude sum).
template <bool Exact>
__global__ void __launch_bounds__(32) cdet_dd_lane(const __grid_constant__ Problem p,
                                                   const __grid_constant__ Scratch w) {
    const int64_t slot = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (slot >= p.batch) return;
    const int64_t c = __ldg(w.config_at + slot);
    const int n = __ldg(p.orders + c);
    const int nmax = p.max_order;
    if (n < 1 || n > nmax) return;
    const int64_t groups = (p.batch + kWarp - 1) / kWarp;
    const DD zero{0.0, 0.0};
    const DD threshold{p.dd_threshold.hi, p.dd_threshold.lo};
    const bool filter = dd_gt(threshold, zero);
    int32_t status = 0;
    DD value[2];
    for (int set = 0; set < 2; ++set) {
        const int r = set == 0 ? 2 : 1;
        if (n == 1) {
            const double* diag = w.diag + c * 2 * 2 * nmax;
            const DD shu{p.dd_shift[0].hi, p.dd_shift[0].lo}, shd{p.dd_shift[1].hi, p.dd_shift[1].lo};
            const DD su = dd_add(DD{diag[(set * 2) * nmax], 0.0}, shu);
            const DD sd = dd_add(DD{diag[(set * 2 + 1) * nmax], 0.0}, shd);
            const DD ru = dd_mul(dd_mul(DD{static_cast<double>(-r), 0.0}, DD{p.dd_u.hi, p.dd_u.lo}),
                                 DD{p.dd_beta.hi, p.dd_beta.lo});
            value[set] = dd_mul(ru, dd_sub(dd_mul(su, sd), dd_mul(shu, shd)));
            continue;
        }
        const DD* a = lane_a(w, slot, set, nmax);
        DD* dp = lane_dp(w, slot, set, nmax, groups);
        dp[0] = a[1 * kWarp];
        const uint32_t rest_limit = 1u << (n - 1);
        for (int bits = 2; bits <= n; ++bits) {
            for (uint32_t rest = (1u << (bits - 1)) - 1u; rest < rest_limit; rest = next_same_popcount(rest)) {
                DD acc = a[static_cast<int64_t>((rest << 1) | 1u) * kWarp];
                if constexpr (Exact) {
                    DD rhs = dd_abs(acc);
                    for (uint32_t sm = (rest - 1u) & rest;; sm = (sm - 1u) & rest) {
                        const DD term = dd_mul(dp[static_cast<int64_t>(sm) * kWarp],
                                               a[static_cast<int64_t>((rest ^ sm) << 1) * kWarp]);
                        acc = dd_sub(acc, term);
                        rhs = dd_add(rhs, dd_abs(term));
                        if (sm == 0) break;
                    }
                    if (filter && dd_lt(dd_abs(acc), dd_mul(threshold, rhs))) acc = zero;
                } else {
                    double rhs = fabs(acc.hi);
                    for (uint32_t sm = (rest - 1u) & rest;; sm = (sm - 1u) & rest) {
                        const DD x = dp[static_cast<int64_t>(sm) * kWarp];
                        const DD y = a[static_cast<int64_t>((rest ^ sm) << 1) * kWarp];
                        const double ph = dmul(x.hi, y.hi);
                        double pe = dfma(x.hi, y.hi, -ph);
                        pe = dfma(x.hi, y.lo, pe);
                        pe = dfma(x.lo, y.hi, pe);
                        double e;
                        const double s = two_sum(acc.hi, -ph, e);
                        e = dadd(e, dsub(acc.lo, pe));
                        acc.hi = quick_two_sum(s, e, acc.lo);
                        rhs = dadd(rhs, fabs(ph));
                        if (sm == 0) break;
                    }
                    if (filter && fabs(acc.hi) < dmul(threshold.hi, rhs)) acc = zero;
                }
                dp[static_cast<int64_t>(rest) * kWarp] = acc;
                if (bits == n) break;  // one mask at the top level
            }
        }
        const DD top = dp[static_cast<int64_t>(rest_limit - 1u) * kWarp];
        value[set] = dd_mul(DD{p.pref_dd[set][n].hi, p.pref_dd[set][n].lo}, top);
        if (!dd_finite(value[set])) status |= kStatusNonFinite;
    }
    const DD result = dd_sub(value[0], dd_mul(DD{2.0, 0.0}, value[1]));
    p.values[c] = dadd(result.hi, result.lo);
    if (status) atomicOr(p.status + c, status);
}

}  // namespace

// Smallest batch that runs the lane form (a warp of configurations per SM).
static int64_t dd_lane_min_batch(int sm_count) { return static_cast<int64_t>(sm_count > 0 ? sm_count : 152) * kWarp; }

cudaError_t launch_integrand_dd(const Problem& p, const Scratch& w, int sm_count, cudaStream_t stream) {
    if (p.batch <= 0) return cudaSuccess;
    const bool two_spins = !(p.same_spin[0] && p.same_spin[1]);
    const bool lanes = p.integrand_form == kIntegrandStaged ||
                       (p.integrand_form == kIntegrandAuto && p.batch >= dd_lane_min_batch(sm_count));
    if (w.dd_lanes && lanes) {
        const size_t ws_bytes = compact_minors_layout(p.max_order, two_spins, true).total * sizeof(DD);
        const int wpb = static_cast<int>(std::max<size_t>(1, std::min<size_t>(kDDMaxWarps, (227 * 1024) / ws_bytes)));
        const int sms = sm_count > 0 ? sm_count : 152;
        const int per_sm = std::max(1, static_cast<int>((227 * 1024) / (ws_bytes * wpb + 1024)));
        int64_t blocks = std::min<int64_t>(static_cast<int64_t>(sms) * per_sm, (p.batch * 2 + wpb - 1) / wpb);
        blocks = std::min<int64_t>(blocks, std::max<int64_t>(1, static_cast<int64_t>(w.ws_warps) / (2 * wpb)));
        const size_t smem = ws_bytes * wpb;
        auto minors = p.fused_cdet ? principal_minors_dd<false> : principal_minors_dd<true>;
        cudaError_t err = cudaFuncSetAttribute(minors, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(smem));
        if (err != cudaSuccess) return err;
        minors<<<static_cast<unsigned>(blocks), wpb * kWarp, smem, stream>>>(p, w);
        err = cudaGetLastError();
        if (err != cudaSuccess) return err;
        // the reference's arithmetic on the FP64 assembly; the lighter one on the split assembly
        // one warp per block, so that a small batch still spreads over every SM
        if (p.fused_cdet)
            cdet_dd_lane<false><<<static_cast<unsigned>((p.batch + kWarp - 1) / kWarp), kWarp, 0, stream>>>(p, w);
        else
            cdet_dd_lane<true><<<static_cast<unsigned>((p.batch + kWarp - 1) / kWarp), kWarp, 0, stream>>>(p, w);
        return cudaGetLastError();
    }
    const size_t ws_bytes = compact_minors_layout(p.max_order, two_spins, true).total * sizeof(DD);
    const size_t budget = 227 * 1024;
    const int wpb = static_cast<int>(std::max<size_t>(1, std::min<size_t>(kDDMaxWarps, budget / ws_bytes)));
    const int sms = sm_count > 0 ? sm_count : 152;
    const int per_sm = std::max(1, static_cast<int>(budget / (ws_bytes * wpb + 1024)));
    int64_t blocks = static_cast<int64_t>(sms) * per_sm;
    // each warp takes two warps' LU-fallback regions of the scratch
    blocks = std::min<int64_t>(blocks, std::max<int64_t>(1, static_cast<int64_t>(w.ws_warps) / (2 * wpb)));
    blocks = std::min<int64_t>(blocks, (p.batch + wpb - 1) / wpb);
    const size_t smem = ws_bytes * wpb;
    cudaError_t err = cudaFuncSetAttribute(integrand_dd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(smem));
    if (err != cudaSuccess) return err;
    integrand_dd<<<static_cast<unsigned>(blocks), wpb * kWarp, smem, stream>>>(p, w);
    return cudaGetLastError();
}

}  // namespace cdet
