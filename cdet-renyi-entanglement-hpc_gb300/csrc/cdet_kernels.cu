// FP64 CDet integrand kernels for sm_103a.
//
// Three launches per batch of vertex configurations:
//
//  1. green_assembly_fp64: one thread per Green-matrix entry (configuration,
//     table set, i, j). It decodes the two vertices, forms the lookup
//     descriptor and evaluates the 2-D Chebyshev sum of the spin-up (and, when
//     the tables differ, spin-down) block by the reference's Clenshaw
//     recurrences, rows in descending order with the outer recurrence fused.
//  2. principal_minors_fp64: one warp per (configuration, table set). The
//     warp runs the shifted Schur-complement recursion of mat2pm level by
//     level, lanes spread over (set, row, column) work items, then the prefix
//     product and the shift removal, and writes a[mask] = pm_up * pm_down into
//     a lane-interleaved array for step 3.
//  3. cdet_fp64: one lane per configuration, 32 configurations per warp. Each
//     lane runs the connected-sum recursion of its configuration serially, in
//     the reference's mask and submask order, so the FP64 pipe always runs
//     full warps. It then applies the prefactors and forms
//     twisted - 2 * ordinary.
//
// On GB300 the FP64 pipe retires about 504 G lane-operations per second and a
// partially active warp costs as much as a full one, so all three kernels keep
// every lane of every FP64 instruction busy.
#include "cdet_device.cuh"
#include "cdet_kernels.cuh"

#include <algorithm>

namespace cdet {

namespace {

// sampled_coordinate_to_index (g_funcs.h:315-342) on value*extent; flags
// values the reference would reject (non-finite, outside the int range).
__device__ __forceinline__ int coordinate_index(double scaled, int extent, bool& bad) {
    if (!(scaled > -2147483648.0 && scaled < 2147483648.0)) {
        bad = true;
        return 0;
    }
    int index = static_cast<int>(floor(scaled));
    if (index < 0) index = 0;
    if (index >= extent) index = extent - 1;
    return index;
}

struct Vertex {
    double tau, tau_unit;
    int x, y, replica;
};

// Vertex decode of integrand_temp_typed (integrand_replica_randomly_sampled.h:422-432).
__device__ __forceinline__ Vertex decode_vertex(const double* __restrict__ v, const Scalars& s,
                                                int replica_count, bool& bad) {
    Vertex out;
    const double tu = __ldg(v + 0);
    if (!isfinite(tu)) bad = true;
    out.tau_unit = tu;
    out.tau = dmul(s.beta, tu);
    out.x = coordinate_index(dmul(static_cast<double>(s.n1), __ldg(v + 1)), s.n1, bad);
    out.y = coordinate_index(dmul(static_cast<double>(s.n2), __ldg(v + 2)), s.n2, bad);
    out.replica = replica_count <= 1
                      ? 0
                      : coordinate_index(dmul(static_cast<double>(replica_count), __ldg(v + 3)),
                                         replica_count, bad);
    return out;
}

__device__ __forceinline__ double clamp_unit(double value) {
    if (value < -1.0) return -1.0;
    if (value > 1.0) return 1.0;
    return value;
}

// ------------------------------------------------------ 1. assembly -------
// Entry (i, j) of table set `set` of configuration c (order n): decode,
// descriptor, Clenshaw sums, shifts and scale. With copy_retained, a pair of
// vertices retained from the previous evaluation is copied instead.
__device__ __forceinline__ void assemble_entry(const Problem& p, const Scratch& w, int64_t c, int set, int i, int j,
                                               int n, bool copy_retained) {
    const int nmax = p.max_order;
    const int64_t per_set = static_cast<int64_t>(nmax) * nmax;
    const Scalars& s = p.s;
    const int replica_count = set == 0 ? 2 : 1;
    bool bad = false;
    const double* vbase = p.vertices + c * static_cast<int64_t>(nmax) * 4;
    const Vertex vi = decode_vertex(vbase + 4 * i, s, replica_count, bad);
    const Vertex vj = decode_vertex(vbase + 4 * j, s, replica_count, bad);
    if (bad) {
        atomicOr(p.status + c, kStatusBadInput);
        return;
    }
    if (copy_retained && copy_reused_pair(p, w.green, w.diag, c, set, i, j, n)) return;

    // prepare_green_lookup_descriptor (g_funcs.h:609-653).
    const bool upper = (i != j) && (vi.tau_unit > vj.tau_unit);
    const uint64_t sitepair =
        ((((static_cast<uint64_t>(vi.replica) * 2u + static_cast<uint64_t>(vj.replica)) * s.n1 +
           vi.x) * s.n2 + vi.y) * s.n1 + vj.x) * s.n2 + vj.y;
    const double t_outer = upper ? vi.tau : vj.tau;  // the later time of the pair
    const double t_inner = upper ? vj.tau : vi.tau;
    const TableDev& tu = p.up[set];
    const TableDev& td = p.down[set];
    const bool one_spin = p.same_spin[set] != 0;
    double up, down;
    if (t_outer < s.branch_eps) {
        up = __ldg((upper ? tu.upper_corners : tu.lower_corners) + sitepair);
        down = one_spin ? up : __ldg((upper ? td.upper_corners : td.lower_corners) + sitepair);
    } else {
        const double u = clamp_unit(dsub(ddiv(dmul(2.0, t_outer), s.beta), 1.0));
        const double v = clamp_unit(dsub(ddiv(dmul(2.0, t_inner), t_outer), 1.0));
        const uint64_t base = sitepair * static_cast<uint64_t>(s.nu) * static_cast<uint64_t>(s.nv);
        const double* bu = (upper ? tu.upper : tu.lower) + base;
        OuterClenshaw ou;
        ou.init(s.nu - 1, u);
        if (one_spin) {
            for (int a = s.nu - 1; a >= 0; --a)
                ou.push(a, clenshaw_row(bu + static_cast<int64_t>(a) * s.nv, s.nv - 1, v));
            up = down = ou.result();
        } else {
            const double* bd = (upper ? td.upper : td.lower) + base;
            OuterClenshaw od;
            od.init(s.nu - 1, u);
            for (int a = s.nu - 1; a >= 0; --a) {
                double ru, rd;
                clenshaw_row_pair(bu + static_cast<int64_t>(a) * s.nv,
                                  bd + static_cast<int64_t>(a) * s.nv, s.nv - 1, v, ru, rd);
                ou.push(a, ru);
                od.push(a, rd);
            }
            up = ou.result();
            down = od.result();
        }
    }
    // fill_pair_range (integrand_replica_randomly_sampled.h:467-473).
    const int64_t mslot = (c * 2 + set) * 2;
    if (i == j) {
        const double up_raw = up, down_raw = down;
        up = dadd(up, s.diag_up_shift);
        down = dadd(down, s.diag_down_shift);
        // the double-double order-1 branch adds its own shifts to the unshifted value
        w.diag[mslot * nmax + i] = p.raw_diag ? up_raw : up;
        w.diag[(mslot + 1) * nmax + i] = p.raw_diag ? down_raw : down;
    }
    w.green[mslot * per_set + i * n + j] = dmul(up, s.scale);
    w.green[(mslot + 1) * per_set + i * n + j] = dmul(down, s.scale);
}

// One thread per (configuration, set, i, j) entry.
__global__ void __launch_bounds__(128) green_assembly_fp64(const __grid_constant__ Problem p,
                                                          const __grid_constant__ Scratch w) {
    const int nmax = p.max_order;
    const int64_t per_set = static_cast<int64_t>(nmax) * nmax;
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= p.batch * 2 * per_set) return;
    const int64_t c = idx / (2 * per_set);
    const int64_t rem = idx - c * 2 * per_set;
    const int set = static_cast<int>(rem / per_set);
    const int pair = static_cast<int>(rem - set * per_set);
    const int i = pair / nmax;
    const int j = pair - i * nmax;
    const int n = p.all_subsets ? nmax : __ldg(p.orders + c);
    if (n < 1 || n > nmax) {
        if (rem == 0) atomicOr(p.status + c, kStatusBadInput);
        return;
    }
    if (i >= n || j >= n) return;
    assemble_entry(p, w, c, set, i, j, n, p.reuse_mask != nullptr);
}

// Green-pair reuse in the FP64 assembly (all-subsets batches): the copies and
// the evaluations go to separate launches, so no warp waits on another lane's
// Clenshaw sums while its own lanes only copy. reuse_offsets: per
// configuration the first of its fresh entries, 2 (n^2 - k^2) of them with k
// retained vertices, exclusive over configurations, and the total.
constexpr uint32_t kReuseTotalIndex = 56;  // the total's uint32 slot in Scratch::order_count

__global__ void __launch_bounds__(1024) reuse_scan(const __grid_constant__ Problem p, int32_t* offsets,
                                                   uint32_t* total) {
    __shared__ uint32_t part[1024];
    const int n = p.max_order;
    const int64_t per = (p.batch + 1023) / 1024;
    const int64_t begin = threadIdx.x * per, end = min(p.batch, begin + per);
    uint32_t sum = 0;
    for (int64_t c = begin; c < end; ++c) {
        const int k = __popcll(__ldg(p.reuse_mask + c));
        sum += 2u * static_cast<uint32_t>(n * n - k * k);
    }
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {  // inclusive scan of the thread sums
        const uint32_t add = threadIdx.x >= static_cast<unsigned>(off) ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += add;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - sum;
    for (int64_t c = begin; c < end; ++c) {
        offsets[c] = static_cast<int32_t>(run);
        const int k = __popcll(__ldg(p.reuse_mask + c));
        run += 2u * static_cast<uint32_t>(n * n - k * k);
    }
    if (threadIdx.x == 1023) *total = part[1023];
}

// The copies: one thread per entry of the retained block (i, j < k).
__global__ void __launch_bounds__(128) green_copy_retained(const __grid_constant__ Problem p,
                                                          const __grid_constant__ Scratch w) {
    const int n = p.max_order;
    const int64_t per_set = static_cast<int64_t>(n) * n;
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= p.batch * 2 * per_set) return;
    const int64_t c = idx / (2 * per_set);
    const int64_t rem = idx - c * 2 * per_set;
    const int set = static_cast<int>(rem / per_set);
    const int pair = static_cast<int>(rem - set * per_set);
    const int i = pair / n, j = pair - (pair / n) * n;
    const int k = __popcll(__ldg(p.reuse_mask + c));
    if (i >= k || j >= k) return;
    bool bad = false;  // the decode's checks, so the status bits are a fresh evaluation's
    const double* vbase = p.vertices + c * n * 4;
    decode_vertex(vbase + 4 * i, p.s, set == 0 ? 2 : 1, bad);
    decode_vertex(vbase + 4 * j, p.s, set == 0 ? 2 : 1, bad);
    if (bad) {
        atomicOr(p.status + c, kStatusBadInput);
        return;
    }
    copy_reused_pair(p, w.green, w.diag, c, set, i, j, n);
}

// The evaluations: one thread per fresh entry, compacted over the batch.
// Fresh entries of a set, in order: rows i < k at columns k..n-1, then rows
// i >= k at every column.
__global__ void __launch_bounds__(128) green_assembly_fp64_fresh(const __grid_constant__ Problem p,
                                                                const __grid_constant__ Scratch w,
                                                                const int32_t* __restrict__ offsets,
                                                                const uint32_t* __restrict__ total) {
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= static_cast<int64_t>(__ldg(total))) return;
    // the configuration: the last offset <= idx
    int64_t lo = 0, hi = p.batch - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (static_cast<int64_t>(__ldg(offsets + mid)) <= idx) lo = mid;
        else hi = mid - 1;
    }
    const int64_t c = lo;
    const int n = p.max_order;
    const int k = __popcll(__ldg(p.reuse_mask + c));
    const int per = n * n - k * k;  // fresh entries per set (> 0 here: this configuration owns idx)
    const int r = static_cast<int>(idx - __ldg(offsets + c));
    const int set = r >= per ? 1 : 0;
    const int rr = r - set * per;
    int i, j;
    if (rr < k * (n - k)) {
        i = rr / (n - k);
        j = k + (rr - i * (n - k));
    } else {
        const int q = rr - k * (n - k);
        i = k + q / n;
        j = q - (q / n) * n;
    }
    assemble_entry(p, w, c, set, i, j, n, false);
}

// ------------------------------------------------- 2. principal minors ----
// Partial-pivot LU minor of the principal submatrix selected by mask
// (determinant_principal_minor_from_buffer, fast_principle_minors.h:39-105);
// m is this lane's n*n scratch.
__device__ double minor_by_lu(const double* a, int n, uint32_t mask, double* m) {
    int idx[kMaxOrder];
    int k = 0;
    for (int i = 0; i < n; ++i)
        if (mask & (1u << i)) idx[k++] = i;
    if (k == 0) return 1.0;
    for (int r = 0; r < k; ++r)
        for (int c = 0; c < k; ++c) m[r * k + c] = a[idx[r] * n + idx[c]];
    double det = 1.0;
    int sign = 1;
    for (int col = 0; col < k; ++col) {
        int pivot_row = col;
        double pivot_abs = fabs(m[col * k + col]);
        for (int row = col + 1; row < k; ++row) {
            const double cand = fabs(m[row * k + col]);
            if (cand > pivot_abs) {
                pivot_abs = cand;
                pivot_row = row;
            }
        }
        if (pivot_abs == 0.0) return 0.0;
        if (pivot_row != col) {
            for (int c = col; c < k; ++c) {
                const double t = m[col * k + c];
                m[col * k + c] = m[pivot_row * k + c];
                m[pivot_row * k + c] = t;
            }
            sign = -sign;
        }
        const double pivot = m[col * k + col];
        det = dmul(det, pivot);
        for (int row = col + 1; row < k; ++row) {
            const double factor = ddiv(m[row * k + col], pivot);
            if (factor == 0.0) continue;
            m[row * k + col] = 0.0;
            for (int c = col + 1; c < k; ++c)
                m[row * k + c] = dfma(-factor, m[col * k + c], m[row * k + c]);
        }
    }
    return sign < 0 ? -det : det;
}

// The shift removal of mat2pm (fast_principle_minors.h:230-243) for
// 2^11..2^14 minors, blocked so that each value is read and written twice
// instead of once per bit: first the bits above 9, a column of 2^(n-10)
// values per lane in registers, then bits 9..0 on chunks of 1,024 values (32
// per lane; bits 5..9 between a lane's registers, bits 0..4 across lanes by
// shuffles). Every value takes the same fma(-p, partner, value) updates in
// the same (descending-bit) order as the unblocked loop, so the minors are
// bit for bit the same.
template <int HighBits>
__device__ __forceinline__ void remove_shift_high(double* shifted, double p, int lane) {
    constexpr int kCount = 1 << HighBits;
    for (uint32_t c = lane; c < 1024u; c += kWarp) {
        double r[kCount];
#pragma unroll
        for (int k = 0; k < kCount; ++k) r[k] = shifted[c + 1024u * k];
#pragma unroll
        for (int b = HighBits - 1; b >= 0; --b)
#pragma unroll
            for (int k = 0; k < kCount; ++k)
                if (k & (1 << b)) r[k] = dfma(-p, r[k ^ (1 << b)], r[k]);
#pragma unroll
        for (int k = 0; k < kCount; ++k) shifted[c + 1024u * k] = r[k];
    }
}

__device__ __forceinline__ void remove_shift_blocked(double* shifted, int n, double p, int lane) {
    switch (n) {  // n = 11..14
        case 11: remove_shift_high<1>(shifted, p, lane); break;
        case 12: remove_shift_high<2>(shifted, p, lane); break;
        case 13: remove_shift_high<3>(shifted, p, lane); break;
        case 14: remove_shift_high<4>(shifted, p, lane); break;
        default: break;
    }
    __syncwarp();
    const uint32_t subsets = 1u << n;
    for (uint32_t h = 0; h < subsets; h += 1024u) {
        double r[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) r[j] = shifted[h + lane + kWarp * j];
#pragma unroll
        for (int b = 4; b >= 0; --b)  // bits 9..5: between registers
#pragma unroll
            for (int j = 0; j < 32; ++j)
                if (j & (1 << b)) r[j] = dfma(-p, r[j ^ (1 << b)], r[j]);
#pragma unroll
        for (int b = 4; b >= 0; --b) {  // bits 4..0: across lanes
            const int m = 1 << b;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const double v = __shfl_xor_sync(0xffffffffu, r[j], m);
                if (lane & m) r[j] = dfma(-p, v, r[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) shifted[h + lane + kWarp * j] = r[j];
    }
    __syncwarp();
}

// mat2pm_from_buffer (fast_principle_minors.h:120-246) for one matrix, by a
// whole warp. On return shifted[mask] (mask >= 1) holds the principal minor
// of the rows/columns in mask. Returns true when a pivot sent the matrix to
// the whole-matrix LU fallback (which this function then also runs). With
// the compact layout (lay.arena > 0) the level lists live in shifted's arena
// (compact_minors_layout), and each shifted minor is written once as p + its
// pivot entry, the value the initialise-then-add form gives.
__device__ bool mat2pm_warp(const double* A, int n, double tol, double shift_param,
                            const WsLayout& lay, double* ws, double* shifted, double* lu_lane,
                            int lane) {
    const int msize = n * n;
    const uint32_t subsets = 1u << n;
    double max_abs = 0.0;
    for (int k = lane; k < msize; k += kWarp) {
        const double e = fabs(A[k]);
        if (e > max_abs) max_abs = e;
    }
    for (int off = 16; off > 0; off >>= 1) {
        const double o = __shfl_xor_sync(0xffffffffu, max_abs, off);
        if (o > max_abs) max_abs = o;
    }
    const bool explicit_shift = !(shift_param < 0.0);
    const double p = explicit_shift ? shift_param : ddiv(max_abs, static_cast<double>(msize));
    if (max_abs == 0.0 && p == 0.0) {
        for (uint32_t m = lane; m < subsets; m += kWarp) shifted[m] = 0.0;
        __syncwarp();
        return false;
    }
    const double fallback_eps = (tol > 0.0 && max_abs > 0.0) ? dmul(tol, max_abs) : 0.0;

    // A node's pivot inverse replaces its pivot entry and its first-column
    // factors replace column 0 of rows 1.. (the children take only rows and
    // columns 1.., and the first minor has read the pivot entry already), so
    // the recursion needs no space besides its two lists.
    const bool compact = lay.arena > 0;
    double* old_list = compact ? shifted + compact_list_offset(n, 0, lay.arena) : ws + lay.old_list;
    double* new_list = compact ? nullptr : ws + lay.new_list;
    for (int k = lane; k < msize; k += kWarp) old_list[k] = A[k];
    if (compact) {
        if (lane == 0) shifted[0] = 1.0;
    } else {
        for (uint32_t m = lane; m < subsets; m += kWarp) shifted[m] = m == 0 ? 1.0 : p;
    }
    __syncwarp();
    if (lane == 0) shifted[1] = dadd(compact ? p : shifted[1], old_list[0]);

    uint32_t minor_index = 2;
    bool fell_back = false;
    for (int level = 0; level < n - 1; ++level) {
        const int old_size = n - level;
        const int old_msize = old_size * old_size;
        const int new_size = old_size - 1;
        const int new_msize = new_size * new_size;
        const int sets = 1 << level;
        // pivots of this level, one per set
        bool bad_pivot = false;
        for (int set = lane; set < sets; set += kWarp) {
            const double pivot = dadd(old_list[set * old_msize], p);
            const double pa = fabs(pivot);
            if (pa == 0.0 || (fallback_eps > 0.0 && pa <= fallback_eps)) bad_pivot = true;
            // 1.0 / pivot, correctly rounded (IEEE): the same value
            old_list[set * old_msize] = __drcp_rn(pivot);
        }
        if (__any_sync(0xffffffffu, bad_pivot)) {
            fell_back = true;
            break;
        }
        __syncwarp();
        // first-column factors, one per (set, row), in place of the column
        for (int item = lane; item < sets * new_size; item += kWarp) {
            const int set = item / new_size;
            const int row = item - set * new_size;
            double* entry = old_list + set * old_msize + (row + 1) * old_size;
            *entry = dmul(*entry, old_list[set * old_msize]);
        }
        __syncwarp();
        if (compact) {
            if (level == n - 2) {
                // the last level's 1 x 1 children, straight to their shifted minors
                for (int set = lane; set < sets; set += kWarp) {
                    const double* m = old_list + set * 4;
                    const double base = m[3];
                    shifted[minor_index + set] = dadd(p, base);
                    shifted[minor_index + sets + set] = dadd(p, dfma(-m[1], m[2], base));
                }
                __syncwarp();
                minor_index += 2 * sets;
                break;
            }
            new_list = shifted + compact_list_offset(n, level + 1, lay.arena);
        }
        // submatrix without the pivot, and its Schur complement
        const int items = sets * new_msize;
#pragma unroll 4
        for (int item = lane; item < items; item += kWarp) {  // independent items, several in flight
            const int set = item / new_msize;
            const int e = item - set * new_msize;
            const int row = e / new_size;
            const int col = e - row * new_size;
            const int src = set * old_msize;
            const double base = old_list[src + (row + 1) * old_size + col + 1];
            new_list[item] = base;
            new_list[items + item] = dfma(-old_list[src + 1 + col], old_list[src + (row + 1) * old_size], base);
        }
        __syncwarp();
        for (int m = lane; m < 2 * sets; m += kWarp)
            shifted[minor_index + m] = dadd(compact ? p : shifted[minor_index + m], new_list[m * new_msize]);
        minor_index += 2 * sets;
        double* t = old_list;
        old_list = new_list;
        new_list = t;
        __syncwarp();
    }
    if (fell_back) {
        // determinant_principal_minors_from_buffer (fast_principle_minors.h:107-115)
        for (uint32_t m = 1 + lane; m < subsets; m += kWarp) shifted[m] = minor_by_lu(A, n, m, lu_lane);
        __syncwarp();
        return true;
    }
    // prefix product over levels
    for (uint32_t step = 1; step < subsets; step <<= 1) {
#pragma unroll 4
        for (uint32_t set = step + 1 + lane; set < 2 * step; set += kWarp)
            shifted[set] = dmul(shifted[set], shifted[set - step]);
        __syncwarp();
    }
    // remove the uniform shift by multilinearity
    if (n >= 11 && n <= 14) {  // (at order 10 the unblocked loop on shared memory is faster)
        remove_shift_blocked(shifted, n, p, lane);
        return false;
    }
    for (uint32_t step = subsets; step > 1; step >>= 1) {
        const uint32_t half = step >> 1;
        const int hb = __ffs(half) - 1;  // half = 2^hb: the element's bit hb is set, its partner's clear
#pragma unroll 4
        for (uint32_t q = lane; q < subsets / 2; q += kWarp) {
            const uint32_t ss = ((q >> hb) << (hb + 1)) + half + (q & (half - 1u));
            shifted[ss] = dfma(-p, shifted[ss - half], shifted[ss]);
        }
        __syncwarp();
    }
    return false;
}

// ---- orders 11..14: the Schur recursion in chunks of subtrees ----------
// The whole-level lists of these orders (up to 2 x 18,432 doubles at order
// 14) do not fit shared memory, and in the global workspace every level
// streams them through DRAM. Here only the top T levels run breadth-first
// in the warp's global workspace (small lists); the 2^T nodes of level T are
// then taken G at a time, and each group's subtrees run breadth-first in
// shared memory. A node's pivot, factors and Schur complement depend only on
// its parent, and each shifted minor receives its one addition, so every
// value is the whole-level recursion's bit for bit; the same pivots are
// checked, so the LU fallback is taken exactly when it is there.
struct ChunkGeom {
    int T, log2g;     // chunk level and log2 of the nodes per chunk
    int list, aux;    // doubles of one chunk list buffer and of the chunk's pivot/factor buffer
    __host__ __device__ int doubles() const { return 2 * list + aux; }
};

__host__ __device__ inline ChunkGeom chunk_geom(int n) {
    ChunkGeom g;
    g.T = n <= 11 ? 4 : (n <= 13 ? 5 : 6);
    g.log2g = 2;
    const int G = 1 << g.log2g, m = n - g.T;
    int list = 0, aux = 0;
    for (int j = 0; j < m; ++j) list = max(list, (G << j) * (m - j) * (m - j));
    for (int j = 0; j + 1 < m; ++j) aux = max(aux, (G << j) * (m - j));  // pivots' inverses + factors
    g.list = (list + 1) & ~1;
    g.aux = (aux + 1) & ~1;
    return g;
}

constexpr int kChunkMinOrder = 11, kChunkMaxOrder = 14;

// The FP64 minors' workspace of a batch of orders up to nmax: the aux region
// only where the chunked recursion can run (mat2pm_warp needs none).
__host__ __device__ inline WsLayout fp64_minors_layout(int nmax, bool two_spins) {
    return ws_layout(nmax, two_spins, nmax >= kChunkMinOrder);
}

// The FP64 warp minors' workspace: compact up to order 10 in shared memory,
// else the list layout above.
__host__ __device__ inline WsLayout minors_layout(int nmax, bool two_spins, bool shared) {
    return shared && nmax <= kCompactMaxOrder ? compact_minors_layout(nmax, two_spins)
                                              : fp64_minors_layout(nmax, two_spins);
}

// Shared doubles per warp of the chunked minors for a batch of orders up to nmax.
__host__ __device__ inline int chunk_doubles_upto(int nmax) {
    int d = 0;
    for (int n = kChunkMinOrder; n <= min(nmax, kChunkMaxOrder); ++n) d = max(d, chunk_geom(n).doubles());
    return d;
}

// One level of the shifted Schur recursion on `nodes` matrices of old_size^2
// in old_list, writing their 2 * nodes children (old_size - 1)^2 to new_list:
// the first `nodes` without the pivot row and column, the next `nodes` the
// Schur complements (mat2pm_from_buffer, fast_principle_minors.h:165-215).
// Child q's shifted minor is shifted[base + index(q)], index(q) = c0 + (q mod
// G) + (q div G) * 2^T (G = 2^log2g): the identity for whole levels (c0 = 0,
// log2g = 30), the global node numbers of a chunk's subtrees otherwise.
// Returns false when a pivot sends the matrix to the LU fallback. Each
// shifted minor receives exactly one addition, p + the child's pivot entry,
// written directly (the whole-level form adds it to the p it initialised).
__device__ bool schur_level(const double* old_list, double* new_list, double* inv, int nodes, int old_size,
                            double p, double fallback_eps, double* shifted, uint32_t base, uint32_t c0,
                            int log2g, int T, int lane) {
    const int old_msize = old_size * old_size;
    const int new_size = old_size - 1;
    const int new_msize = new_size * new_size;
    bool bad_pivot = false;
    for (int set = lane; set < nodes; set += kWarp) {
        const double pivot = dadd(old_list[set * old_msize], p);
        const double pa = fabs(pivot);
        if (pa == 0.0 || (fallback_eps > 0.0 && pa <= fallback_eps)) bad_pivot = true;
        inv[set] = __drcp_rn(pivot);  // 1.0 / pivot, correctly rounded (IEEE): the same value
    }
    if (__any_sync(0xffffffffu, bad_pivot)) return false;
    __syncwarp();
    double* factor = inv + nodes;
    for (int item = lane; item < nodes * new_size; item += kWarp) {
        const int set = item / new_size;
        const int row = item - set * new_size;
        factor[item] = dmul(old_list[set * old_msize + (row + 1) * old_size], inv[set]);
    }
    __syncwarp();
    const int items = nodes * new_msize;
    for (int item = lane; item < items; item += kWarp) {
        const int set = item / new_msize;
        const int e = item - set * new_msize;
        const int row = e / new_size;
        const int col = e - row * new_size;
        const int src = set * old_msize;
        const double b = old_list[src + (row + 1) * old_size + col + 1];
        new_list[item] = b;
        new_list[items + item] = dfma(-old_list[src + 1 + col], factor[set * new_size + row], b);
    }
    __syncwarp();
    const uint32_t gmask = (1u << log2g) - 1u;
    for (int q = lane; q < 2 * nodes; q += kWarp) {
        const uint32_t idx = base + c0 + (static_cast<uint32_t>(q) & gmask) +
                             ((static_cast<uint32_t>(q) >> log2g) << T);
        shifted[idx] = dadd(p, new_list[q * new_msize]);
    }
    __syncwarp();
    return true;
}

// The prefix product of mat2pm (fast_principle_minors.h:217-228) on a global
// array: shifted[step + 1 + t] *= shifted[1 + t], eight elements per lane in
// flight.
__device__ __forceinline__ void prefix_product_global(double* shifted, uint32_t subsets, int lane) {
    for (uint32_t step = 2; step < subsets; step <<= 1) {
        const uint32_t count = step - 1;
        for (uint32_t t0 = 0; t0 < count; t0 += 8 * kWarp) {
            double x[8], y[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t t = t0 + u * kWarp + lane;
                x[u] = t < count ? shifted[step + 1 + t] : 0.0;
                y[u] = t < count ? shifted[1 + t] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t t = t0 + u * kWarp + lane;
                if (t < count) shifted[step + 1 + t] = dmul(x[u], y[u]);
            }
        }
        __syncwarp();
    }
}

// mat2pm_warp for orders 11..14 with the chunked recursion: the top levels'
// lists in the global workspace ws, the chunks' in `chunk` (shared memory,
// chunk_geom(n).doubles()), the shifted minors in global memory.
__device__ bool mat2pm_chunked(const double* A, int n, double tol, double shift_param, const WsLayout& lay,
                               double* ws, double* shifted, double* lu_lane, double* chunk, int lane) {
    const int msize = n * n;
    const uint32_t subsets = 1u << n;
    double max_abs = 0.0;
    for (int k = lane; k < msize; k += kWarp) {
        const double e = fabs(A[k]);
        if (e > max_abs) max_abs = e;
    }
    for (int off = 16; off > 0; off >>= 1) {
        const double o = __shfl_xor_sync(0xffffffffu, max_abs, off);
        if (o > max_abs) max_abs = o;
    }
    const bool explicit_shift = !(shift_param < 0.0);
    const double p = explicit_shift ? shift_param : ddiv(max_abs, static_cast<double>(msize));
    if (max_abs == 0.0 && p == 0.0) {
        for (uint32_t m = lane; m < subsets; m += kWarp) shifted[m] = 0.0;
        __syncwarp();
        return false;
    }
    const double fallback_eps = (tol > 0.0 && max_abs > 0.0) ? dmul(tol, max_abs) : 0.0;
    double* old_list = ws + lay.old_list;
    double* new_list = ws + lay.new_list;
    double* inv = ws + lay.aux;
    for (int k = lane; k < msize; k += kWarp) old_list[k] = A[k];
    // every shifted minor from 2 on is written once by its node below
    if (lane == 0) {
        shifted[0] = 1.0;
        shifted[1] = dadd(p, A[0]);
    }
    __syncwarp();
    const ChunkGeom g = chunk_geom(n);
    bool ok = true;
    for (int level = 0; level < g.T && ok; ++level) {
        ok = schur_level(old_list, new_list, inv, 1 << level, n - level, p, fallback_eps, shifted,
                         2u << level, 0u, 30, 0, lane);
        double* t = old_list;
        old_list = new_list;
        new_list = t;
    }
    // old_list: the 2^T matrices of level T, (n - T)^2 each
    const int m = n - g.T, msz = m * m, G = 1 << g.log2g;
    for (uint32_t c0 = 0; ok && c0 < (1u << g.T); c0 += G) {
        double* co = chunk;
        double* cn = chunk + g.list;
        double* caux = chunk + 2 * g.list;
        for (int k = lane; k < G * msz; k += kWarp) co[k] = old_list[c0 * msz + k];
        __syncwarp();
        for (int j = 0; j + 1 < m && ok; ++j) {
            ok = schur_level(co, cn, caux, G << j, m - j, p, fallback_eps, shifted, 2u << (g.T + j), c0,
                             g.log2g, g.T, lane);
            double* t = co;
            co = cn;
            cn = t;
        }
    }
    if (!ok) {
        // determinant_principal_minors_from_buffer (fast_principle_minors.h:107-115)
        for (uint32_t mk = 1 + lane; mk < subsets; mk += kWarp) shifted[mk] = minor_by_lu(A, n, mk, lu_lane);
        __syncwarp();
        return true;
    }
    prefix_product_global(shifted, subsets, lane);
    remove_shift_blocked(shifted, n, p, lane);
    return false;
}

// use_smem: 1 = the whole workspace in shared memory; 0 = in the global
// workspace; 2 = chunked (orders 11..14): lists of the chunks in shared
// memory, the top levels' lists and the shifted minors in the global workspace.
__global__ void __launch_bounds__(384) principal_minors_fp64(const __grid_constant__ Problem p,
                                                            const __grid_constant__ Scratch w,
                                                            int use_smem) {
    extern __shared__ double smem[];
    const int lane = threadIdx.x & (kWarp - 1);
    const int warp_in_block = threadIdx.x / kWarp;
    const int warps_per_block = blockDim.x / kWarp;
    const int64_t global_warp = static_cast<int64_t>(blockIdx.x) * warps_per_block + warp_in_block;
    const int64_t total_warps = static_cast<int64_t>(gridDim.x) * warps_per_block;
    const int nmax = p.max_order;
    // the global workspace is laid out for two spins; shared memory for what
    // the sets need, compact up to order 10 (A then read from the Green matrices)
    const WsLayout lay = minors_layout(nmax, use_smem != 1 || !(p.same_spin[0] && p.same_spin[1]), use_smem == 1);
    double* ws = use_smem == 1 ? smem + static_cast<size_t>(warp_in_block) * lay.total
                               : w.ws_global + static_cast<size_t>(global_warp) * lay.total;
    double* lu_lane = w.lu_scratch + (static_cast<size_t>(global_warp) * kWarp + lane) * nmax * nmax;
    double* chunk = use_smem == 2 ? smem + static_cast<size_t>(warp_in_block) * chunk_doubles_upto(nmax) : nullptr;
    auto minors = [&](const double* A, int n, double* shifted) {
        return (chunk && n >= kChunkMinOrder && n <= kChunkMaxOrder)
                   ? mat2pm_chunked(A, n, p.s.tol_fpm, p.s.fpm_shift, lay, ws, shifted, lu_lane, chunk, lane)
                   : mat2pm_warp(A, n, p.s.tol_fpm, p.s.fpm_shift, lay, ws, shifted, lu_lane, lane);
    };
    const uint32_t full = 1u << nmax;
    const int64_t items = p.batch * 2;
    for (int64_t item = global_warp; item < items; item += total_warps) {
        const int64_t c = item >> 1;
        const int set = static_cast<int>(item & 1);
        const int n = p.all_subsets ? nmax : __ldg(p.orders + c);
        if (n < 2 || n > nmax) continue;  // order 1 needs no minors; bad orders are flagged by step 1
        const double* green = w.green + (c * 2 + set) * 2 * static_cast<int64_t>(nmax) * nmax;
        bool fb = false;
        const bool one_spin = p.same_spin[set] != 0;
        if (lay.arena > 0) {
            fb |= minors(green, n, ws + lay.shifted_up);
            if (!one_spin) fb |= minors(green + static_cast<int64_t>(nmax) * nmax, n, ws + lay.shifted_down);
        } else {
            double* A = ws + lay.a;
            for (int k = lane; k < n * n; k += kWarp) A[k] = green[k];
            __syncwarp();
            fb |= minors(A, n, ws + lay.shifted_up);
            if (!one_spin) {
                for (int k = lane; k < n * n; k += kWarp) A[k] = green[static_cast<int64_t>(nmax) * nmax + k];
                __syncwarp();
                fb |= minors(A, n, ws + lay.shifted_down);
            }
        }
        const double* su = ws + lay.shifted_up;
        const double* sd = one_spin ? su : ws + lay.shifted_down;
        // a[mask] = up[mask-1] * down[mask-1] (integrand_replica_randomly_sampled.h:254-257)
        const int64_t slot = p.sorted ? __ldg(w.slot_of + c) : c;  // lane-interleaved position
        double* a = w.a_int + ((slot >> 5) * 2 + set) * static_cast<int64_t>(full) * kWarp + (slot & 31);
        for (uint32_t m0 = 0; m0 < (1u << n); m0 += 8 * kWarp) {  // eight products per lane in flight
            double x[8], y[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t m = m0 + u * kWarp + lane;
                x[u] = m < (1u << n) ? su[m] : 0.0;
                y[u] = m < (1u << n) ? sd[m] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t m = m0 + u * kWarp + lane;
                if (m < (1u << n)) a[static_cast<int64_t>(m) * kWarp] = m == 0 ? 0.0 : dmul(x[u], y[u]);
            }
        }
        if (fb && lane == 0) atomicOr(p.status + c, kStatusFpmFallback);
        __syncwarp();
    }
}

// ---------------------------------------------------------- 3. CDet -------
// One pair update of the recursion: acc -= dp[s] a[m \ s] and rhs += |that
// term|. The reference's form rounds the product, the difference and the sum
// separately (bit-identical FP64); the fused form, used behind the split
// assembly whose Green matrices already differ from the FP64 ones at the
// last bits, takes two FMAs (one rounding each, one FP64 operation fewer).
template <bool Fused>
__device__ __forceinline__ void pair_update(double dps, double am, double& acc, double& rhs) {
    if constexpr (Fused) {
        acc = __fma_rn(-dps, am, acc);
        rhs = __fma_rn(fabs(dps), fabs(am), rhs);
    } else {
        const double term = dmul(dps, am);
        acc = dsub(acc, term);
        rhs = dadd(rhs, fabs(term));
    }
}

// compute_dp_ztransform (integrand_replica_randomly_sampled.h:226-290) for
// this lane's configuration: only masks holding vertex 0 are reduced.
template <bool Fused>
__device__ double cdet_single(const double* a, double* dp, int n, double threshold) {
    const bool filter = threshold > 0.0;
    dp[1 * kWarp] = a[1 * kWarp];
    for (int bits = 2; bits <= n; ++bits) {
        // masks = 1 | (rest << 1) with popcount(rest) = bits-1, increasing
        const uint32_t rest_limit = 1u << (n - 1);
        for (uint32_t rest = (1u << (bits - 1)) - 1u; rest < rest_limit; rest = next_same_popcount(rest)) {
            const uint32_t mask = (rest << 1) | 1u;
            double acc = a[mask * kWarp];
            double rhs = fabs(acc);
            // submasks holding vertex 0, in the reference's descending order
            for (uint32_t s = (rest - 1u) & rest;; s = (s - 1u) & rest) {
                const uint32_t sub = (s << 1) | 1u;
                pair_update<Fused>(dp[sub * kWarp], a[(mask ^ sub) * kWarp], acc, rhs);
                if (s == 0) break;
            }
            if (filter && fabs(acc) < dmul(threshold, rhs)) acc = 0.0;
            dp[mask * kWarp] = acc;
            if (bits == n) break;  // only one mask at the top level
        }
    }
    return dp[((1u << n) - 1u) * kWarp];
}

// compute_dp_ztransform_all_subsets (:292-347): every mask, anchored at its
// lowest vertex.
template <bool Fused>
__device__ void cdet_all(const double* a, double* dp, int n, double threshold) {
    const bool filter = threshold > 0.0;
    dp[0] = 0.0;
    for (int i = 0; i < n; ++i) dp[(1u << i) * kWarp] = a[(1u << i) * kWarp];
    const uint32_t limit = 1u << n;
    for (int bits = 2; bits <= n; ++bits) {
        for (uint32_t mask = (1u << bits) - 1u; mask < limit; mask = next_same_popcount(mask)) {
            const uint32_t anchor = mask & (~mask + 1u);
            const uint32_t rest = mask ^ anchor;
            double acc = a[mask * kWarp];
            double rhs = fabs(acc);
            for (uint32_t s = (rest - 1u) & rest;; s = (s - 1u) & rest) {
                const uint32_t sub = s | anchor;
                pair_update<Fused>(dp[sub * kWarp], a[(mask ^ sub) * kWarp], acc, rhs);
                if (s == 0) break;
            }
            if (filter && fabs(acc) < dmul(threshold, rhs)) acc = 0.0;
            dp[mask * kWarp] = acc;
            if (bits == n) break;
        }
    }
}

// order1_density_integrand_from_sampled_vertex (:173-213): shifted diagonal
// values of one vertex -> (-r) U beta (up*down - shift_up*shift_down).
__device__ __forceinline__ double order1_value(const Scalars& s, double su, double sd, int r) {
    const double counter = dmul(s.diag_up_shift, s.diag_down_shift);
    return dmul(dmul(dmul(static_cast<double>(-r), s.u), s.beta), dsub(dmul(su, sd), counter));
}

__global__ void __launch_bounds__(128) cdet_fp64(const __grid_constant__ Problem p,
                                                const __grid_constant__ Scratch w) {
    // one lane per slot; with p.sorted the slots hold the configurations
    // in decreasing order, so the lanes of a warp run recursions of (nearly)
    // equal length
    const int64_t slot = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (slot >= p.batch) return;
    const int64_t c = p.sorted ? __ldg(w.config_at + slot) : slot;
    const int lane = static_cast<int>(slot & 31);
    const int nmax = p.max_order;
    const int64_t full = int64_t{1} << nmax;
    const int n = p.all_subsets ? nmax : __ldg(p.orders + c);
    if (n < 1 || n > nmax) return;
    const Scalars& s = p.s;
    const double threshold = dmul(s.z_eps0, s.z_safety);
    const int64_t g = slot >> 5;
    int32_t status = 0;
    const double* diag = w.diag + c * 2 * 2 * nmax;  // [set][spin][i]

    if (!p.all_subsets) {
        DD value[2];
        for (int set = 0; set < 2; ++set) {
            const int r = set == 0 ? 2 : 1;
            if (n == 1) {
                // order-1 branch (cdet_integrand_evaluator.h:171-201): no finiteness check
                const double raw = order1_value(s, diag[(set * 2) * nmax], diag[(set * 2 + 1) * nmax], r);
                value[set] = DD{raw, 0.0};
            } else {
                const double* a = w.a_int + (g * 2 + set) * full * kWarp + lane;
                double* dp = w.dp_int + (g * 2 + set) * full * kWarp + lane;
                const double cset = p.fused_cdet ? cdet_single<true>(a, dp, n, threshold)
                                                 : cdet_single<false>(a, dp, n, threshold);
                const DDPair pf = p.pref_dd[set][n];
                value[set] = dd_mul(DD{pf.hi, pf.lo}, DD{cset, 0.0});
                if (!dd_finite(value[set])) status |= kStatusNonFinite;
            }
        }
        const DD result = dd_sub(value[0], dd_mul(DD{2.0, 0.0}, value[1]));
        p.values[c] = dadd(result.hi, result.lo);
    } else {
        // integrand_all_subset_values_typed_into (:826-877) per set, then
        // values[mask] -= 2 * ordinary[mask] (cdet_integrand_evaluator.h:346-350)
        double* out = p.values + c * full;
        for (int set = 0; set < 2; ++set) {
            const int r = set == 0 ? 2 : 1;
            const double* a = w.a_int + (g * 2 + set) * full * kWarp + lane;
            double* dp = w.dp_int + (g * 2 + set) * full * kWarp + lane;
            if (p.fused_cdet) cdet_all<true>(a, dp, n, threshold);
            else cdet_all<false>(a, dp, n, threshold);
            const uint32_t count = 1u << n;
            for (uint32_t mask = 0; mask < count; ++mask) {
                const int k = __popc(mask);
                double v;
                if (k == 0) {
                    v = 0.0;
                } else if (k == 1) {
                    const int i = __ffs(mask) - 1;
                    v = order1_value(s, diag[(set * 2) * nmax + i], diag[(set * 2 + 1) * nmax + i], r);
                } else {
                    v = dmul(p.pref_ld[set][k], dp[static_cast<int64_t>(mask) * kWarp]);
                }
                if (!isfinite(v)) status |= kStatusNonFinite;
                if (set == 0) out[mask] = v;
                else out[mask] = dsub(out[mask], dmul(2.0, v));
            }
        }
    }
    if (status) atomicOr(p.status + c, status);
}


// ------------------------------------- 3a'. all-subsets CDet, warp form ----
// compute_dp_ztransform_all_subsets for small batches (a few MCMCMC chains):
// one warp per configuration, both sets at once, a and dp of each set in
// shared memory. The masks of one popcount level are independent; the lanes
// share the level's masks of both sets, dealt out by colex rank so that no
// lane holds more than its share, and each mask's submask sum runs on one
// lane in the reference's descending order with the same operations as
// cdet_all, so the values are those of cdet_fp64 bit for bit. The lane form
// keeps the FP64 pipe full on large batches; this form gives a small batch 32
// lanes per configuration.
template <bool Fused>
__global__ void __launch_bounds__(128) cdet_all_warp(const __grid_constant__ Problem p,
                                                    const __grid_constant__ Scratch w) {
    extern __shared__ double all_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + warp;
    if (c >= p.batch) return;  // whole warps
    const int n = p.max_order;
    const uint32_t count = 1u << n;
    double* base = all_smem + static_cast<size_t>(warp) * 4 * count;  // [set][a, dp][count]
    const Scalars& s = p.s;
    const double threshold = dmul(s.z_eps0, s.z_safety);
    const bool filter = threshold > 0.0;
    const int64_t g = c >> 5;
    const int cl = static_cast<int>(c & 31);
    for (int set = 0; set < 2; ++set) {
        const double* a = w.a_int + (g * 2 + set) * static_cast<int64_t>(count) * kWarp + cl;
        double* a_s = base + set * 2 * count;
        for (uint32_t m = lane; m < count; m += 32) a_s[m] = a[static_cast<int64_t>(m) * kWarp];
    }
    __syncwarp();
    for (int item = lane; item < 2 * n; item += 32) {
        const int set = item >= n ? 1 : 0, i = item - set * n;
        double* a_s = base + set * 2 * count;
        a_s[count + (1u << i)] = a_s[1u << i];  // dp of a singleton
    }
    __syncwarp();
    for (int bits = 2; bits <= n; ++bits) {
        const uint32_t per = kBinomial.c[n][bits];
        for (uint32_t item = lane; item < 2 * per; item += 32) {
            const int set = item >= per ? 1 : 0;
            const uint32_t mask = colex_subset(item - set * per, bits, n);
            const double* a_s = base + set * 2 * count;
            double* dp = base + set * 2 * count + count;
            const uint32_t anchor = mask & (~mask + 1u);
            const uint32_t rest = mask ^ anchor;
            double acc = a_s[mask];
            double rhs = fabs(acc);
            for (uint32_t sm = (rest - 1u) & rest;; sm = (sm - 1u) & rest) {
                const uint32_t sub = sm | anchor;
                pair_update<Fused>(dp[sub], a_s[mask ^ sub], acc, rhs);
                if (sm == 0) break;
            }
            if (filter && fabs(acc) < dmul(threshold, rhs)) acc = 0.0;
            dp[mask] = acc;
        }
        __syncwarp();  // the next level reads this one
    }
    // integrand_all_subset_values_typed_into (:826-877) per set, then
    // twisted - 2 * ordinary (cdet_integrand_evaluator.h:346-350)
    const double* diag = w.diag + c * 2 * 2 * n;
    double* out = p.values + c * static_cast<int64_t>(count);
    bool bad = false;
    for (uint32_t mask = lane; mask < count; mask += 32) {
        const int k = __popc(mask);
        double v[2];
        for (int set = 0; set < 2; ++set) {
            const int r = set == 0 ? 2 : 1;
            if (k == 0) {
                v[set] = 0.0;
            } else if (k == 1) {
                const int i = __ffs(mask) - 1;
                v[set] = order1_value(s, diag[(set * 2) * n + i], diag[(set * 2 + 1) * n + i], r);
            } else {
                v[set] = dmul(p.pref_ld[set][k], base[set * 2 * count + count + mask]);
            }
            if (!isfinite(v[set])) bad = true;
        }
        out[mask] = dsub(v[0], dmul(2.0, v[1]));
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(p.status + c, kStatusNonFinite);
}

// ------------------------------------------------- 3b. CDet, warp form ----
// The single-top recursion behind the split assembly, one warp per
// (configuration, set), a and dp in shared memory. The masks of one popcount
// level are independent; each gets L lanes (a power of two) that split its
// submasks on the L highest set bits and add their partial sums with
// shuffles, so the FP64 pipe sees few idle lanes even at the top levels.
// Each pair update is one FP64 FMA. The round-off filter's magnitude sum
// runs in FP32 on the terms' magnitudes scaled by 2^(-e |m|) (e: binary
// exponent of the first singleton), which keeps all terms of a mask near 1
// whatever the order; each magnitude is formed from the two factors' exponent
// and mantissa bits (product_magnitude), so a pair update loads only its two
// doubles from shared memory. Magnitudes are clamped to the FP32 range, and a
// non-finite accumulator is never zeroed.
constexpr int kWarpCdetMaxOrder = 10;
// warps per block of cdet_split_warp: two blocks of 14 warps (8 KB each at
// order 10) fill an SM's shared memory, 28 warps per SM
constexpr int kWarpCdetWarps = 14;

__device__ const uint16_t kBinom[11][11] = {
    {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {1, 2, 1, 0, 0, 0, 0, 0, 0, 0, 0},
    {1, 3, 3, 1, 0, 0, 0, 0, 0, 0, 0},
    {1, 4, 6, 4, 1, 0, 0, 0, 0, 0, 0},
    {1, 5, 10, 10, 5, 1, 0, 0, 0, 0, 0},
    {1, 6, 15, 20, 15, 6, 1, 0, 0, 0, 0},
    {1, 7, 21, 35, 35, 21, 7, 1, 0, 0, 0},
    {1, 8, 28, 56, 70, 56, 28, 8, 1, 0, 0},
    {1, 9, 36, 84, 126, 126, 84, 36, 9, 1, 0},
    {1, 10, 45, 120, 210, 252, 210, 120, 45, 10, 1}};

// Subset of size m of {0, ..., N-1} with colex rank r, as a bit mask.
__device__ __forceinline__ uint32_t colex_unrank(uint32_t r, int m, int N) {
    uint32_t set = 0;
    int hi = N - 1;
    for (int i = m; i >= 1; --i) {
        int c = i - 1;
        while (c + 1 <= hi && kBinom[c + 1][i] <= r) ++c;
        set |= 1u << c;
        r -= kBinom[c][i];
        hi = c - 1;
    }
    return set;
}

// |x y| 2^(-s) as a float, from the exponent fields and the leading 20
// mantissa bits of x and y (integer work only; the filter's magnitude sums
// need about 2^-20 relative accuracy). field_bias = 127 - 2046 - s. Zeros and
// subnormals give 0; the exponent is clamped so the result stays finite.
__device__ __forceinline__ float product_magnitude(double x, double y, int field_bias) {
    const int hx = __double2hiint(x), hy = __double2hiint(y);
    const float mx = __int_as_float(0x3F800000 | ((hx & 0xFFFFF) << 3));
    const float my = __int_as_float(0x3F800000 | ((hy & 0xFFFFF) << 3));
    const int ex = ((hx >> 20) & 0x7FF), ey = ((hy >> 20) & 0x7FF);
    int field = ex + ey + field_bias;
    field = (ex == 0 || ey == 0) ? 0 : min(max(field, 0), 252);
    return mx * my * __int_as_float(field << 23);
}

// The fused pair updates of one lane: over the submasks sm = fixed | sl of
// rest (sl a subset of low, sm != rest), part += dp[sm] a[rest ^ sm] as FMAs
// and rpart += their scaled magnitudes, with dp and a indexed by mask >> 1.
// The three lowest bits of low are enumerated inside an unrolled block of
// eight terms (independent loads and magnitudes, two alternating FMA chains)
// and the other bits by the outer loop, in a fixed order, so the result is
// deterministic. The excluded submask sm = rest (its dp is this level's, not
// yet written) contributes exact zeros.
// Shared-memory slot of entry x of a warp's a or dp array in cdet_split_warp:
// bits 4..7 folded into the bank bits 0..3, which spreads the lanes' entries
// (masks of one level) over more banks.
__device__ __forceinline__ uint32_t swz(uint32_t x) { return x ^ ((x >> 4) & 15u); }

template <bool Swz>
__device__ __forceinline__ void fused_submask_sum(const double* dp_s, const double* a_s, uint32_t rest,
                                                  uint32_t fixed, uint32_t low, int field_bias, double& part,
                                                  float& rpart) {
    if (__popc(low) < 3) {
        for (uint32_t sl = low;; sl = (sl - 1u) & low) {
            const uint32_t sm = fixed | sl;
            if (sm != rest) {
                const double x = dp_s[Swz ? swz(sm) : sm], y = a_s[Swz ? swz(rest ^ sm) : (rest ^ sm)];
                part = __fma_rn(x, y, part);
                rpart += product_magnitude(x, y, field_bias);
            }
            if (sl == 0) break;
        }
        return;
    }
    const uint32_t b0 = low & (~low + 1u);
    const uint32_t r1 = low ^ b0;
    const uint32_t b1 = r1 & (~r1 + 1u);
    const uint32_t r2 = r1 ^ b1;
    const uint32_t b2 = r2 & (~r2 + 1u);
    const uint32_t hi = r2 ^ b2;
    double p0 = 0.0, p1 = 0.0;
    float m0 = 0.0f, m1 = 0.0f;
    for (uint32_t h = hi;; h = (h - 1u) & hi) {
        const uint32_t base = fixed | h;
#pragma unroll
        for (int j = 7; j >= 0; --j) {
            const uint32_t sm = base | ((j & 4) ? b2 : 0u) | ((j & 2) ? b1 : 0u) | ((j & 1) ? b0 : 0u);
            const bool skip = sm == rest;
            const double x = skip ? 0.0 : dp_s[Swz ? swz(sm) : sm];
            const double y = skip ? 0.0 : a_s[Swz ? swz(rest ^ sm) : (rest ^ sm)];
            if (j & 1) {
                p1 = __fma_rn(x, y, p1);
                m1 += product_magnitude(x, y, field_bias);
            } else {
                p0 = __fma_rn(x, y, p0);
                m0 += product_magnitude(x, y, field_bias);
            }
        }
        if (h == 0) break;
    }
    part = dadd(part, dadd(p1, p0));
    rpart += m1 + m0;
}

// |v| * 2^k as a float, clamped to the finite range (|k| <= 1000).
__device__ __forceinline__ float scaled_magnitude(double v, int k) {
    const double p2 = __longlong_as_double(static_cast<long long>(1023 + k) << 52);
    return fminf(static_cast<float>(fabs(dmul(v, p2))), 3.0e38f);
}

// The fused single-top recursion of one set of one configuration on one warp
// (order n >= 2): a_s[swz(m >> 1)] holds a of the even masks, a_odd[mask *
// stride] a of the odd ones, and dp of the odd masks goes to dp_s[swz(mask >>
// 1)]. Returns dp of the full mask (every lane). cdet_split_warp and the
// queue form both call it, so their values are the same bit for bit.
__device__ __forceinline__ double split_cdet_recursion(const double* a_s, double* dp_s, const double* a_odd,
                                                       int64_t stride, int n, double threshold, int lane) {
    const bool filter = threshold > 0.0;
    const float thresholdf = static_cast<float>(threshold);
    const int count = 1 << n;
    int e = 0;
    {
        const uint64_t bits = static_cast<uint64_t>(__double_as_longlong(a_odd[1 * stride]));
        const int field = static_cast<int>((bits >> 52) & 0x7FF);
        if (field != 0 && field != 0x7FF) e = field - 1023;
        e = e > 90 ? 90 : (e < -90 ? -90 : e);  // |e| * nmax stays within 1000
    }
    if (lane == 0) dp_s[swz(0)] = a_odd[1 * stride];
    __syncwarp();
    const int nbits = n - 1;
    for (int k = 2; k <= n; ++k) {
        const int kk = k - 1;                 // rest = mask >> 1 has kk of nbits bits
        const int masks = kBinom[nbits][kk];
        const int subs = 1 << kk;             // submasks of rest, rest itself included
        for (int base = 0; base < masks;) {
            const int remaining = masks - base;
            int L = 1, take = kWarp;
            if (remaining < kWarp) {
                while (L * 2 * remaining <= kWarp && L * 2 <= subs) L *= 2;
                take = remaining;
                if (4 * L * remaining < 3 * kWarp && L * 2 <= subs) {  // < 75% of lanes busy
                    L *= 2;
                    take = kWarp / L;
                }
            }
            const int q = __ffs(L) - 1;
            const int idx = base + (lane >> q);
            const int j = lane & (L - 1);
            const bool active = (lane >> q) < take && idx < masks;
            double part = 0.0;
            float rpart = 0.0f;
            uint32_t mask = 0;
            const int field_bias = 127 - 2046 - e * k;
            if (active) {
                const uint32_t rest = colex_unrank(static_cast<uint32_t>(idx), kk, nbits);
                mask = (rest << 1) | 1u;
                uint32_t top = 0, low = rest;
                for (int t = 0; t < q; ++t) {
                    const uint32_t hb = 1u << (31 - __clz(low));
                    top |= hb;
                    low ^= hb;
                }
                uint32_t fixed = 0, tb = top;
                for (int t = 0; t < q; ++t) {
                    const uint32_t lb = tb & (~tb + 1u);
                    if ((j >> t) & 1) fixed |= lb;
                    tb ^= lb;
                }
                fused_submask_sum<true>(dp_s, a_s, rest, fixed, low, field_bias, part, rpart);
            }
            for (int off = 1; off < L; off <<= 1) {
                part = dadd(part, __shfl_xor_sync(0xffffffffu, part, off));
                rpart += __shfl_xor_sync(0xffffffffu, rpart, off);
            }
            if (active && j == 0) {
                const double am = a_odd[static_cast<int64_t>(mask) * stride];
                double acc = dsub(am, part);
                const float rhs = scaled_magnitude(am, -e * k) + rpart;
                if (filter && scaled_magnitude(acc, -e * k) < thresholdf * rhs) acc = 0.0;
                dp_s[swz(mask >> 1)] = acc;
            }
            base += take;
        }
        __syncwarp();
    }
    return dp_s[swz((count - 1) >> 1)];
}

__global__ void __launch_bounds__(kWarpCdetWarps * 32, 2) cdet_split_warp(const __grid_constant__ Problem p,
                                                                       const __grid_constant__ Scratch w) {
    extern __shared__ __align__(16) unsigned char cdet_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nmax = p.max_order;
    const int full_n = 1 << nmax;
    // a of the masks without vertex 0 (even; the pair updates' second factor)
    // and dp of the masks with it (odd), both at mask >> 1; a of an odd mask
    // is read once per mask from global memory
    double* a_s = reinterpret_cast<double*>(cdet_smem) + warp * full_n;
    double* dp_s = a_s + full_n / 2;
    const Scalars& s = p.s;
    const double threshold = dmul(s.z_eps0, s.z_safety);
    {  // one configuration per warp: lane cl of 32-configuration group g
        const int64_t c = static_cast<int64_t>(blockIdx.x) * kWarpCdetWarps + warp;
        if (c >= p.batch) return;
        const int64_t g = c >> 5;
        const int cl = static_cast<int>(c & 31);
        const int n = __ldg(p.orders + c);
        if (n < 1 || n > nmax) return;
        const double* diag = w.diag + c * 2 * 2 * nmax;
        int32_t status = 0;
        DD value_twisted{0.0, 0.0}, value_ordinary{0.0, 0.0};
#pragma unroll
        for (int set = 0; set < 2; ++set) {
            const int r = set == 0 ? 2 : 1;
            DD& value = set == 0 ? value_twisted : value_ordinary;
            if (n == 1) {
                value = DD{order1_value(s, diag[(set * 2) * nmax], diag[(set * 2 + 1) * nmax], r), 0.0};
                continue;
            }
            const double* ag = w.a_int + (g * 2 + set) * static_cast<int64_t>(full_n) * kWarp + cl;
            const int count = 1 << n;
            for (int m2 = lane; m2 < count / 2; m2 += kWarp) a_s[swz(m2)] = ag[static_cast<int64_t>(2 * m2) * kWarp];
            __syncwarp();
            const double top = split_cdet_recursion(a_s, dp_s, ag, kWarp, n, threshold, lane);
            const DDPair pf = p.pref_dd[set][n];
            value = dd_mul(DD{pf.hi, pf.lo}, DD{top, 0.0});
            if (!dd_finite(value)) status |= kStatusNonFinite;
            __syncwarp();  // the next set reuses the arrays
        }
        if (lane == 0) {
            const DD result = dd_sub(value_twisted, dd_mul(DD{2.0, 0.0}, value_ordinary));
            p.values[c] = dadd(result.hi, result.lo);
            if (status) atomicOr(p.status + c, status);
        }
    }
}

// ------------------------------ 3c. single-top CDet, block per configuration
// compute_dp_ztransform (integrand_replica_randomly_sampled.h:226-290) for
// orders 11..14, where a batch holds few configurations and a lane's 2^n-entry
// recursion would leave the SMs nearly empty: one CTA per configuration (256
// threads; 512 at n = 14, where the shared memory leaves one CTA per SM),
// a of the masks without vertex 0 and dp of the masks with it
// in shared memory (2^(n-1) doubles each; 128 KiB at n = 14), the masks of
// each popcount level dealt out by colex rank. FP64 form: each mask's
// submask sum runs on one thread in the reference's descending order with
// the reference's operations, so the values are cdet_fp64's bit for bit.
// Fused form (split assembly): the pair updates are FMAs and the round-off
// filter's magnitudes FP32, as in cdet_split_warp; a level with fewer masks
// than threads splits each mask's submasks over a group of L lanes (a fixed
// partition and shuffle order, so the result is deterministic).
constexpr int kBlockCdetMaxOrder = 14;

// colex unranking with the binomials of n <= 13 in shared memory
__device__ __forceinline__ uint32_t colex_subset_s(uint32_t r, int m, int n, const uint32_t (*binom)[16]) {
    uint32_t set = 0;
    int hi = n - 1;
    for (int i = m; i >= 1; --i) {
        int c = hi;
        while (c >= i && binom[c][i] > r) --c;
        set |= 1u << c;
        r -= binom[c][i];
        hi = c - 1;
    }
    return set;
}

// The top levels of the FP64 recursion at order 14 (at most 32 masks of
// 2^12..2^13 terms each): the pair-update products are formed by all threads
// into shared memory, chunk by chunk, and the two serial sums of each mask --
// acc = acc - term and rhs = rhs + |term|, in the reference's submask order --
// run on lane i of two different warps (so on two SM sub-partitions) instead
// of one thread doing product, difference and sum in turn. The same
// operations on the same operands in the same order: bit-identical.
template <int kThreads>
__device__ __forceinline__ void fp64_top_level(const double* ag, const double* a_s, double* dp_s, double* terms,
                                               int terms_capacity, int masks, int kk, int nbits,
                                               const uint32_t (*binom)[16], double threshold, bool filter,
                                               double* chain_rhs) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int total = (1 << kk) - 1;                         // submasks of rest other than rest
    const int chunk = terms_capacity / masks;                // terms per mask per chunk
    const bool chain = warp < 2 && lane < masks;
    uint32_t rest = 0;
    double acc = 0.0, rhs = 0.0;
    if (chain) {
        rest = colex_subset_s(static_cast<uint32_t>(lane), kk, nbits, binom);
        acc = ag[static_cast<int64_t>((rest << 1) | 1u) * kWarp];
        rhs = fabs(acc);
    }
    for (int s0 = 0; s0 < total; s0 += chunk) {
        const int len = min(chunk, total - s0);
        // the products of this chunk: term j of mask i at terms[j * masks + i]
        for (int e = tid; e < len * masks; e += kThreads) {
            const int j = e / masks, i = e - j * masks;
            const uint32_t r = colex_subset_s(static_cast<uint32_t>(i), kk, nbits, binom);
            // the (s0 + j)-th submask in descending order: deposit the bits
            // of 2^kk - 2 - (s0 + j) into the set bits of r
            uint32_t x = static_cast<uint32_t>((1 << kk) - 2 - (s0 + j)), bits = r, sl = 0;
            while (bits) {
                const uint32_t lb = bits & (~bits + 1u);
                if (x & 1u) sl |= lb;
                x >>= 1;
                bits ^= lb;
            }
            terms[j * masks + i] = dmul(dp_s[sl], a_s[r ^ sl]);
        }
        __syncthreads();
        if (chain) {
            if (warp == 0) {
                for (int j = 0; j < len; ++j) acc = dsub(acc, terms[j * masks + lane]);
            } else {
                for (int j = 0; j < len; ++j) rhs = dadd(rhs, fabs(terms[j * masks + lane]));
            }
        }
        __syncthreads();
    }
    if (chain && warp == 1) chain_rhs[lane] = rhs;
    __syncthreads();
    if (chain && warp == 0) {
        if (filter && fabs(acc) < dmul(threshold, chain_rhs[lane])) acc = 0.0;
        dp_s[rest] = acc;  // dp of mask (rest << 1) | 1, at mask >> 1
    }
}

template <bool Fused, int kBlockCdetThreads>
__global__ void __launch_bounds__(kBlockCdetThreads) cdet_block(const __grid_constant__ Problem p,
                                                                const __grid_constant__ Scratch w) {
    extern __shared__ __align__(16) unsigned char cdet_smem[];
    __shared__ uint32_t binom[16][16];
    __shared__ double chain_rhs[kWarp];
    const int tid = threadIdx.x;
    const int nmax = p.max_order;
    const int half = 1 << (nmax - 1);
    double* a_s = reinterpret_cast<double*>(cdet_smem);  // a of even masks, at mask >> 1
    double* dp_s = a_s + half;                           // dp of odd masks, at mask >> 1
    // FP64 form at order 14: the top levels' products (see fp64_top_level)
    constexpr bool kChains = !Fused && kBlockCdetThreads == 512;
    double* terms = dp_s + half;
    const int64_t slot = blockIdx.x;
    const int64_t c = p.sorted ? __ldg(w.config_at + slot) : slot;
    const int64_t g = slot >> 5;
    const int cl = static_cast<int>(slot & 31);
    const int n = __ldg(p.orders + c);
    if (n < 1 || n > nmax) return;  // the whole block
    if (tid < 16 * 16) {
        const int nn = tid >> 4, kk = tid & 15;
        binom[nn][kk] = (nn <= 24 && kk <= nn) ? kBinomial.c[nn][kk] : 0u;
    }
    const Scalars& s = p.s;
    const double threshold = dmul(s.z_eps0, s.z_safety);
    const bool filter = threshold > 0.0;
    const float thresholdf = static_cast<float>(threshold);
    const int64_t full = int64_t{1} << nmax;
    const double* diag = w.diag + c * 2 * 2 * nmax;
    int32_t status = 0;
    DD value[2] = {DD{0.0, 0.0}, DD{0.0, 0.0}};
    for (int set = 0; set < 2; ++set) {
        const int r = set == 0 ? 2 : 1;
        if (n == 1) {
            value[set] = DD{order1_value(s, diag[(set * 2) * nmax], diag[(set * 2 + 1) * nmax], r), 0.0};
            continue;
        }
        const double* ag = w.a_int + (g * 2 + set) * full * kWarp + cl;
        const int count = 1 << n;
        int e = 0;
        if constexpr (Fused) {
            const uint64_t bits = static_cast<uint64_t>(__double_as_longlong(ag[1 * kWarp]));
            const int field = static_cast<int>((bits >> 52) & 0x7FF);
            if (field != 0 && field != 0x7FF) e = field - 1023;
            e = e > 60 ? 60 : (e < -60 ? -60 : e);  // |e| * n stays within 1000
        }
        for (int m2 = tid; m2 < count / 2; m2 += kBlockCdetThreads) a_s[m2] = ag[static_cast<int64_t>(2 * m2) * kWarp];
        if (tid == 0) dp_s[0] = ag[1 * kWarp];
        __syncthreads();
        const int nbits = n - 1;
        for (int k = 2; k <= n; ++k) {
            const int kk = k - 1;            // rest = mask >> 1 has kk of nbits bits
            const int masks = static_cast<int>(binom[nbits][kk]);
            const int subs = 1 << kk;        // submasks of rest, rest itself included
            if constexpr (kChains) {
                if (masks <= kWarp && subs >= 1024) {
                    fp64_top_level<kBlockCdetThreads>(ag, a_s, dp_s, terms, half, masks, kk, nbits, binom,
                                                      threshold, filter, chain_rhs);
                    __syncthreads();
                    continue;
                }
            }
            const int field_bias = 127 - 2046 - e * k;
            for (int base = 0; base < masks;) {
                const int remaining = masks - base;
                int L = 1, take = kBlockCdetThreads;
                if (Fused && remaining < kBlockCdetThreads) {
                    while (L * 2 * remaining <= kBlockCdetThreads && L * 2 <= subs && L < kWarp) L *= 2;
                    take = remaining;
                    if (4 * L * remaining < 3 * kBlockCdetThreads && L * 2 <= subs && L < kWarp) {
                        L *= 2;  // < 75% of the threads busy
                        take = kBlockCdetThreads / L;
                    }
                }
                const int q = __ffs(L) - 1;
                const int idx = base + (tid >> q);
                const bool active = (tid >> q) < take && idx < masks;
                if constexpr (!Fused) {
                    if (active) {
                        const uint32_t rest = colex_subset_s(static_cast<uint32_t>(idx), kk, nbits, binom);
                        const uint32_t mask = (rest << 1) | 1u;
                        double acc = ag[static_cast<int64_t>(mask) * kWarp];
                        double rhs = fabs(acc);
                        for (uint32_t sl = (rest - 1u) & rest;; sl = (sl - 1u) & rest) {
                            const uint32_t sub = (sl << 1) | 1u;
                            pair_update<false>(dp_s[sub >> 1], a_s[(mask ^ sub) >> 1], acc, rhs);
                            if (sl == 0) break;
                        }
                        if (filter && fabs(acc) < dmul(threshold, rhs)) acc = 0.0;
                        dp_s[mask >> 1] = acc;
                    }
                } else {
                    const int j = tid & (L - 1);
                    double part = 0.0;
                    float rpart = 0.0f;
                    uint32_t mask = 0;
                    if (active) {
                        const uint32_t rest = colex_subset_s(static_cast<uint32_t>(idx), kk, nbits, binom);
                        mask = (rest << 1) | 1u;
                        // the top q bits of rest are fixed by the lane's index in its group
                        uint32_t top = 0, low = rest;
                        for (int t = 0; t < q; ++t) {
                            const uint32_t hb = 1u << (31 - __clz(low));
                            top |= hb;
                            low ^= hb;
                        }
                        uint32_t fixed = 0, tb = top;
                        for (int t = 0; t < q; ++t) {
                            const uint32_t lb = tb & (~tb + 1u);
                            if ((j >> t) & 1) fixed |= lb;
                            tb ^= lb;
                        }
                        fused_submask_sum<false>(dp_s, a_s, rest, fixed, low, field_bias, part, rpart);
                    }
                    for (int off = 1; off < L; off <<= 1) {
                        part = dadd(part, __shfl_xor_sync(0xffffffffu, part, off));
                        rpart += __shfl_xor_sync(0xffffffffu, rpart, off);
                    }
                    if (active && j == 0) {
                        const double am = ag[static_cast<int64_t>(mask) * kWarp];
                        double acc = dsub(am, part);
                        const float rhs = scaled_magnitude(am, -e * k) + rpart;
                        if (filter && scaled_magnitude(acc, -e * k) < thresholdf * rhs) acc = 0.0;
                        dp_s[mask >> 1] = acc;
                    }
                }
                base += take;
            }
            __syncthreads();
        }
        if (tid == 0) {
            const DDPair pf = p.pref_dd[set][n];
            value[set] = dd_mul(DD{pf.hi, pf.lo}, DD{dp_s[(count - 1) >> 1], 0.0});
            if (!dd_finite(value[set])) status |= kStatusNonFinite;
        }
        __syncthreads();  // the next set reuses the arrays
    }
    if (tid == 0) {
        const DD result = dd_sub(value[0], dd_mul(DD{2.0, 0.0}, value[1]));
        p.values[c] = dadd(result.hi, result.lo);
        if (status) atomicOr(p.status + c, status);
    }
}

// ------------------------------------------ 4. persistent queue form -------
// Minors, CDet and combine of each configuration in one persistent kernel,
// with no global a array between them. The warps take configurations from
// the order-sorted slots (decreasing order: the longest recursions start
// first, the short ones fill the tail) through an atomic queue head, `grab`
// slots at a time. One warp per configuration (both sets in turn) or a pair
// of warps (one set each, meeting at a named barrier). A warp's shared-memory
// region is the minors workspace; after a set's Schur recursion its lists are
// free and hold the CDet arrays: a of the odd masks replaces the shifted
// minors in place, a of the even masks and dp of the odd ones take the two
// list regions (each holds at least 2^(n-1) doubles: the last Schur level has
// 2^(n-1) lists of one entry). Every set goes through the staged form's
// operations (mat2pm_warp, a = up * down, split_cdet_recursion or the
// reference's descending submask sums), so the values are the staged form's
// bit for bit.

// compute_dp_ztransform (integrand_replica_randomly_sampled.h:226-290) on one
// warp, for order n >= 2: a[mask] for every mask, dp of the odd masks into
// dp_s[mask >> 1]. The masks of a popcount level are dealt to the lanes by
// colex rank; each mask's submask sum runs on one lane in the reference's
// descending order with the reference's operations, so the result is
// cdet_single's bit for bit.
__device__ double fp64_single_warp(const double* a, double* dp_s, int n, double threshold, int lane) {
    const bool filter = threshold > 0.0;
    if (lane == 0) dp_s[0] = a[1];
    __syncwarp();
    const int nbits = n - 1;
    for (int k = 2; k <= n; ++k) {
        const int kk = k - 1;
        const int masks = kBinom[nbits][kk];
        for (int idx = lane; idx < masks; idx += kWarp) {
            const uint32_t rest = colex_unrank(static_cast<uint32_t>(idx), kk, nbits);
            double acc = a[(rest << 1) | 1u];
            double rhs = fabs(acc);
            for (uint32_t sm = (rest - 1u) & rest;; sm = (sm - 1u) & rest) {
                pair_update<false>(dp_s[sm], a[(rest ^ sm) << 1], acc, rhs);
                if (sm == 0) break;
            }
            if (filter && fabs(acc) < dmul(threshold, rhs)) acc = 0.0;
            dp_s[rest] = acc;
        }
        __syncwarp();  // the next level reads this one
    }
    return dp_s[(1u << nbits) - 1u];
}

// One set of configuration c (order n) on one warp: the prefactored value of
// that set; status collects the FPM-fallback and non-finite bits.
template <bool Fused>
__device__ __forceinline__ DD queue_set_value(const Problem& p, const Scratch& w, int64_t c, int set, int n,
                                              const WsLayout& lay, double* ws, double* lu_lane, int lane,
                                              int32_t& status) {
    const Scalars& s = p.s;
    const int nmax = p.max_order;
    if (n == 1) {  // the order-1 branch: no minors, no finiteness check
        const double* diag = w.diag + c * 2 * 2 * nmax;
        return DD{order1_value(s, diag[(set * 2) * nmax], diag[(set * 2 + 1) * nmax], set == 0 ? 2 : 1), 0.0};
    }
    const double* green = w.green + (c * 2 + set) * 2 * static_cast<int64_t>(nmax) * nmax;
    const bool compact = lay.arena > 0;  // A read from the Green matrices, else copied in
    double* A = compact ? nullptr : ws + lay.a;
    bool fb = false;
    if (!compact) {
        for (int k = lane; k < n * n; k += kWarp) A[k] = green[k];
        __syncwarp();
    }
    double* su = ws + lay.shifted_up;
    fb |= mat2pm_warp(compact ? green : A, n, s.tol_fpm, s.fpm_shift, lay, ws, su, lu_lane, lane);
    const bool one_spin = p.same_spin[set] != 0;
    if (!one_spin) {
        const double* green_down = green + static_cast<int64_t>(nmax) * nmax;
        if (!compact) {
            for (int k = lane; k < n * n; k += kWarp) A[k] = green_down[k];
            __syncwarp();
        }
        fb |= mat2pm_warp(compact ? green_down : A, n, s.tol_fpm, s.fpm_shift, lay, ws, ws + lay.shifted_down,
                          lu_lane, lane);
    }
    const double* sd = one_spin ? su : ws + lay.shifted_down;
    const uint32_t count = 1u << n;
    const double threshold = dmul(s.z_eps0, s.z_safety);
    double top;
    if constexpr (Fused) {
        // a = up * down (integrand_replica_randomly_sampled.h:254-257): the
        // even masks to the first list region (swizzled like cdet_split_warp's),
        // the odd ones in place
        double* a_even = ws + lay.new_list;
        for (uint32_t m = lane; m < count; m += kWarp) {
            const double am = m == 0 ? 0.0 : dmul(su[m], sd[m]);
            if (m & 1u) su[m] = am;
            else a_even[swz(m >> 1)] = am;
        }
        __syncwarp();
        top = split_cdet_recursion(a_even, ws + lay.old_list, su, 1, n, threshold, lane);
    } else {
        for (uint32_t m = lane; m < count; m += kWarp) su[m] = m == 0 ? 0.0 : dmul(su[m], sd[m]);
        __syncwarp();
        top = fp64_single_warp(su, ws + lay.old_list, n, threshold, lane);
    }
    const DDPair pf = p.pref_dd[set][n];
    const DD value = dd_mul(DD{pf.hi, pf.lo}, DD{top, 0.0});
    if (!dd_finite(value)) status |= kStatusNonFinite;
    if (fb) status |= kStatusFpmFallback;
    __syncwarp();  // the next set reuses the workspace
    return value;
}

__device__ __forceinline__ void pair_barrier(int pair) {
    asm volatile("bar.sync %0, 64;" ::"r"(pair + 1) : "memory");
}

template <bool Fused, bool Pair>
__global__ void __launch_bounds__(384) integrand_queue(const __grid_constant__ Problem p,
                                                      const __grid_constant__ Scratch w, int grab) {
    extern __shared__ double queue_smem[];
    const int lane = threadIdx.x & (kWarp - 1);
    const int warp_in_block = threadIdx.x / kWarp;
    const int warps_per_block = blockDim.x / kWarp;
    const int64_t global_warp = static_cast<int64_t>(blockIdx.x) * warps_per_block + warp_in_block;
    const int nmax = p.max_order;
    const WsLayout lay = minors_layout(nmax, !(p.same_spin[0] && p.same_spin[1]), true);
    double* ws = queue_smem + static_cast<size_t>(warp_in_block) * lay.total;
    double* lu_lane = w.lu_scratch + (static_cast<size_t>(global_warp) * kWarp + lane) * nmax * nmax;
    uint32_t* head = w.order_count + kQueueHeadIndex;
    const uint32_t batch = static_cast<uint32_t>(p.batch);
    // pair exchange (after the workspaces): [pair] {first slot, status, value hi, value lo}
    const int pair = warp_in_block >> 1, set_of_warp = warp_in_block & 1;
    double* exchange = queue_smem + static_cast<size_t>(warps_per_block) * lay.total + pair * 4;
    for (;;) {
        uint32_t first = 0;
        if constexpr (Pair) {
            if (set_of_warp == 0 && lane == 0)
                reinterpret_cast<uint32_t*>(exchange)[0] = atomicAdd(head, static_cast<uint32_t>(grab));
            pair_barrier(pair);
            first = reinterpret_cast<const volatile uint32_t*>(exchange)[0];
            pair_barrier(pair);  // both warps hold the slot before the next pop
        } else {
            if (lane == 0) first = atomicAdd(head, static_cast<uint32_t>(grab));
            first = __shfl_sync(0xffffffffu, first, 0);
        }
        if (first >= batch) break;
        const uint32_t last = min(first + static_cast<uint32_t>(grab), batch);
        for (uint32_t slot = first; slot < last; ++slot) {
            const int64_t c = __ldg(w.config_at + slot);
            const int n = __ldg(p.orders + c);
            if (n < 1 || n > nmax) continue;  // flagged by the assembly
            int32_t status = 0;
            if constexpr (Pair) {
                const DD v = queue_set_value<Fused>(p, w, c, set_of_warp, n, lay, ws, lu_lane, lane, status);
                if (lane == 0 && set_of_warp == 1) {
                    exchange[2] = v.hi;
                    exchange[3] = v.lo;
                }
                if (lane == 0 && status) atomicOr(p.status + c, status);
                pair_barrier(pair);
                if (lane == 0 && set_of_warp == 0) {
                    const DD ordinary{exchange[2], exchange[3]};
                    const DD result = dd_sub(v, dd_mul(DD{2.0, 0.0}, ordinary));
                    p.values[c] = dadd(result.hi, result.lo);
                }
                pair_barrier(pair);  // the exchange is read before the next write
            } else {
                const DD twisted = queue_set_value<Fused>(p, w, c, 0, n, lay, ws, lu_lane, lane, status);
                const DD ordinary = queue_set_value<Fused>(p, w, c, 1, n, lay, ws, lu_lane, lane, status);
                if (lane == 0) {
                    const DD result = dd_sub(twisted, dd_mul(DD{2.0, 0.0}, ordinary));
                    p.values[c] = dadd(result.hi, result.lo);
                    if (status) atomicOr(p.status + c, status);
                }
            }
        }
    }
}
}  // namespace

size_t minors_workspace_doubles(int max_order) { return ws_layout(max_order).total; }

// Warps of the minors kernel whose workspaces fit one block's shared memory
// (at most kMinorsMaxWarps); the kernel uses shared memory when this is at least 4.
static int minors_warps_in_shared_memory(int max_order, bool two_spins) {
    const size_t ws_bytes = minors_layout(max_order, two_spins, true).total * sizeof(double);
    const size_t smem_budget = 227 * 1024;
    return static_cast<int>(std::min<size_t>(kMinorsMaxWarps, smem_budget / ws_bytes));
}

bool minors_use_global_workspace(int max_order, bool two_spins) {
    return minors_warps_in_shared_memory(max_order, two_spins) < 4;
}

bool fp64_single_order_uses_dp_lanes(int max_order) {
    // orders 11..14 run the block CDet (a and dp in shared memory)
    return !(max_order > kWarpCdetMaxOrder && max_order <= kBlockCdetMaxOrder);
}

cudaError_t launch_fp64_assembly_only(const Problem& p, const Scratch& w, cudaStream_t stream) {
    if (p.batch <= 0) return cudaSuccess;
    const int64_t entries = p.batch * 2 * static_cast<int64_t>(p.max_order) * p.max_order;
    green_assembly_fp64<<<static_cast<unsigned>((entries + 127) / 128), 128, 0, stream>>>(p, w);
    return cudaGetLastError();
}

// ------------------------------------------- order-sorted slots ----------
// A counting sort of a mixed-order batch by decreasing order (invalid orders
// last): config_at[slot] and slot_of[config]. Slots within one order follow
// the atomics' arrival, which changes no value: every configuration is
// computed by the same operations wherever it sits.
__global__ void order_count(const int32_t* __restrict__ orders, int64_t batch, int max_order, uint32_t* count) {
    for (int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; c < batch;
         c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int n = __ldg(orders + c);
        const int b = (n < 1 || n > max_order) ? max_order + 1 : max_order - n;  // bucket 0: the top order
        atomicAdd(count + b, 1u);
    }
}

__global__ void order_scan(uint32_t* count, int buckets) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint32_t run = 0;
    for (int b = 0; b < buckets; ++b) {
        const uint32_t k = count[b];
        count[b] = run;  // first slot of the bucket, then its next free slot
        run += k;
    }
}

__global__ void order_scatter(const int32_t* __restrict__ orders, int64_t batch, int max_order, uint32_t* next,
                              int32_t* __restrict__ slot_of, int32_t* __restrict__ config_at) {
    for (int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; c < batch;
         c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int n = __ldg(orders + c);
        const int b = (n < 1 || n > max_order) ? max_order + 1 : max_order - n;
        const uint32_t slot = atomicAdd(next + b, 1u);
        slot_of[c] = static_cast<int32_t>(slot);
        config_at[slot] = static_cast<int32_t>(c);
    }
}

size_t scratch_bytes(int64_t batch, int max_order, size_t ws_warps, ScratchRegions regions) {
    const size_t groups = static_cast<size_t>((batch + 31) / 32);
    const size_t n2 = static_cast<size_t>(max_order) * max_order;
    const size_t subsets = static_cast<size_t>(1) << max_order;
    size_t total = 0;
    total += static_cast<size_t>(batch) * 4 * n2;                   // green
    total += static_cast<size_t>(batch) * 4 * max_order;            // diag
    total += (regions.dp_lanes ? 2 : 1) * groups * 2 * subsets * kWarp;  // a_int, dp_int
    if (regions.minors_workspace) total += ws_warps * minors_workspace_doubles(max_order);  // minors workspace
    total += ws_warps * kWarp * n2;                                 // LU fallback scratch
    total += 2 * ((static_cast<size_t>(batch) * 4 + 7) / 8) + 32;   // order-sorted slots, buckets
    if (regions.dd_lanes) total += 3 * groups * 2 * subsets * kWarp;  // double-double a and dp
    return total * sizeof(double) + 64 * (regions.dd_lanes ? 10 : 9);
}

void carve_scratch(void* base, int64_t batch, int max_order, size_t ws_warps, Scratch* out,
                   ScratchRegions regions) {
    const size_t groups = static_cast<size_t>((batch + 31) / 32);
    const size_t n2 = static_cast<size_t>(max_order) * max_order;
    const size_t subsets = static_cast<size_t>(1) << max_order;
    char* cursor = static_cast<char*>(base);
    auto take = [&](size_t doubles) {
        double* ptr = reinterpret_cast<double*>(cursor);
        cursor += ((doubles * sizeof(double) + 63) / 64) * 64;
        return ptr;
    };
    out->green = take(static_cast<size_t>(batch) * 4 * n2);
    out->diag = take(static_cast<size_t>(batch) * 4 * max_order);
    out->a_int = take(groups * 2 * subsets * kWarp);
    out->dp_int = regions.dp_lanes ? take(groups * 2 * subsets * kWarp) : nullptr;
    out->ws_global = regions.minors_workspace ? take(ws_warps * minors_workspace_doubles(max_order)) : nullptr;
    out->lu_scratch = take(ws_warps * kWarp * n2);
    out->ws_warps = ws_warps;
    out->slot_of = reinterpret_cast<int32_t*>(take((static_cast<size_t>(batch) * 4 + 7) / 8));
    out->config_at = reinterpret_cast<int32_t*>(take((static_cast<size_t>(batch) * 4 + 7) / 8));
    out->order_count = reinterpret_cast<uint32_t*>(take(32));
    out->dd_lanes = regions.dd_lanes ? take(3 * groups * 2 * subsets * kWarp) : nullptr;
}

// Sort, minors and CDet (or the queue kernel) on the Green matrices in scratch.
static cudaError_t post_assembly(const Problem& p_in, const Scratch& w, int sm_count, cudaStream_t stream,
                                 const KernelEvents* events) {
    Problem p = p_in;
    p.sorted = sorts_orders(p) ? 1 : 0;
    auto mark = [&](int k) {
        if (events && events->marks[k]) cudaEventRecord(events->marks[k], stream);
    };
    const int threads = 128;
    cudaError_t err = cudaSuccess;
    if (p.sorted) {
        const int buckets = p.max_order + 2;
        const unsigned grid = static_cast<unsigned>(std::min<int64_t>((p.batch + 255) / 256, 4 * 152));
        err = cudaMemsetAsync(w.order_count, 0, 64 * sizeof(uint32_t), stream);  // buckets, queue head
        if (err != cudaSuccess) return err;
        order_count<<<grid, 256, 0, stream>>>(p.orders, p.batch, p.max_order, w.order_count);
        order_scan<<<1, 32, 0, stream>>>(w.order_count, buckets);
        order_scatter<<<grid, 256, 0, stream>>>(p.orders, p.batch, p.max_order, w.order_count, w.slot_of,
                                                w.config_at);
        err = cudaGetLastError();
        if (err != cudaSuccess) return err;
    }

    if (p.dd_mode) {
        err = launch_integrand_dd(p, w, sm_count, stream);
        if (err != cudaSuccess) return err;
        mark(3);
        mark(4);
        return cudaSuccess;
    }

    if (uses_queue_form(p)) {
        int wpb = 0, blocks = 0;
        size_t smem = 0;
        queue_launch_shape(p, w, sm_count, &wpb, &blocks, &smem);
        auto kernel = p.fused_cdet ? (p.queue.pair ? integrand_queue<true, true> : integrand_queue<true, false>)
                                   : (p.queue.pair ? integrand_queue<false, true> : integrand_queue<false, false>);
        err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (err != cudaSuccess) return err;
        kernel<<<static_cast<unsigned>(blocks), wpb * kWarp, smem, stream>>>(p, w, std::max(1, p.queue.grab));
        err = cudaGetLastError();
        if (err != cudaSuccess) return err;
        mark(3);
        mark(4);
        return cudaSuccess;
    }

    // Minors: the per-warp workspace goes to shared memory when at least four
    // warps' worth fits a block (one block per SM, as many warps as fit, at
    // most 16; the compact arena up to order 10; without the spin-down minors
    // when both sets have one spin), otherwise to the global workspace (4
    // warps per block).
    const bool two_spins = !(p.same_spin[0] && p.same_spin[1]);
    const size_t ws_bytes = minors_layout(p.max_order, two_spins, true).total * sizeof(double);
    const int fit = minors_warps_in_shared_memory(p.max_order, two_spins);
    const bool use_smem = fit >= 4;
    // orders 11..14 in the global workspace: the chunked recursion, eight
    // warps per block, as many blocks per SM as their chunk buffers allow
    const bool chunked = !use_smem && p.max_order >= kChunkMinOrder && p.max_order <= kChunkMaxOrder;
    const size_t chunk_bytes = chunked ? chunk_doubles_upto(p.max_order) * sizeof(double) : 0;
    const int warps_per_block = use_smem ? fit : (chunked ? 8 : 4);
    const int64_t items = p.batch * 2;
    int64_t blocks = (items + warps_per_block - 1) / warps_per_block;
    const int64_t max_blocks = static_cast<int64_t>(w.ws_warps) / warps_per_block;
    blocks = std::min<int64_t>(blocks, std::max<int64_t>(1, max_blocks));
    const int sms = sm_count > 0 ? sm_count : 152;
    if (use_smem) blocks = std::min<int64_t>(blocks, sms);  // one wave
    if (chunked) {
        const int64_t per_sm = std::max<int64_t>(1, (227 * 1024) / (chunk_bytes * warps_per_block + 1024));
        blocks = std::min<int64_t>(blocks, per_sm * sms);  // one wave
    }
    const size_t smem = use_smem ? ws_bytes * warps_per_block : chunk_bytes * warps_per_block;
    if (smem > 48 * 1024) {
        err = cudaFuncSetAttribute(principal_minors_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(smem));
        if (err != cudaSuccess) return err;
    }
    principal_minors_fp64<<<static_cast<unsigned>(blocks), warps_per_block * kWarp, smem, stream>>>(
        p, w, use_smem ? 1 : (chunked ? 2 : 0));
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    mark(3);

    if (p.fused_cdet && !p.all_subsets && p.max_order <= kWarpCdetMaxOrder) {
        // split assembly: warp-per-configuration recursion in shared memory
        const size_t csmem = static_cast<size_t>(kWarpCdetWarps) * sizeof(double) * (size_t{1} << p.max_order);
        err = cudaFuncSetAttribute(cdet_split_warp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(csmem));
        if (err != cudaSuccess) return err;
        cdet_split_warp<<<static_cast<unsigned>((p.batch + kWarpCdetWarps - 1) / kWarpCdetWarps),
                          kWarpCdetWarps * kWarp, csmem, stream>>>(p, w);
    } else if (p.all_subsets && p.max_order <= kAllWarpMaxOrder && p.all_subsets_form != kFormLane &&
               (p.all_subsets_form == kFormWarp ||
                p.batch < static_cast<int64_t>(all_subsets_lane_form_min_batch(sm_count)))) {
        // a small batch of all-subset envelopes: one warp per configuration,
        // one warp per block while that spreads the batch over more SMs
        const size_t per_warp = 4 * (size_t{1} << p.max_order) * sizeof(double);
        const int warps = p.batch < 4 * static_cast<int64_t>(sm_count > 0 ? sm_count : 152)
                              ? 1
                              : static_cast<int>(std::min<size_t>(4, (200 * 1024) / per_warp));
        const size_t csmem = per_warp * warps;
        if (p.fused_cdet) {
            err = cudaFuncSetAttribute(cdet_all_warp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(csmem));
            if (err != cudaSuccess) return err;
            cdet_all_warp<true><<<static_cast<unsigned>((p.batch + warps - 1) / warps), warps * kWarp, csmem,
                                  stream>>>(p, w);
        } else {
            err = cudaFuncSetAttribute(cdet_all_warp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(csmem));
            if (err != cudaSuccess) return err;
            cdet_all_warp<false><<<static_cast<unsigned>((p.batch + warps - 1) / warps), warps * kWarp, csmem,
                                   stream>>>(p, w);
        }
    } else if (!p.all_subsets && p.max_order > kWarpCdetMaxOrder && p.max_order <= kBlockCdetMaxOrder) {
        // orders 11..14: one block per configuration (slots in decreasing order)
        const bool wide = p.max_order == kBlockCdetMaxOrder;
        // a and dp, plus (FP64 form at order 14) as much again / 2 for the top levels' products
        const size_t csmem = sizeof(double) * (size_t{1} << p.max_order) * (wide && !p.fused_cdet ? 3 : 2) / 2;
        auto kernel = p.fused_cdet ? (wide ? cdet_block<true, 512> : cdet_block<true, 256>)
                                   : (wide ? cdet_block<false, 512> : cdet_block<false, 256>);
        err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(csmem));
        if (err != cudaSuccess) return err;
        kernel<<<static_cast<unsigned>(p.batch), wide ? 512 : 256, csmem, stream>>>(p, w);
    } else {
        cdet_fp64<<<static_cast<unsigned>((p.batch + threads - 1) / threads), threads, 0, stream>>>(p, w);
    }
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    mark(4);
    return cudaSuccess;
}


bool uses_queue_form(const Problem& p) {
    return !p.dd_mode && p.integrand_form == kIntegrandQueue && !p.all_subsets && p.max_order >= 1 &&
           p.max_order <= kQueueMaxOrder;
}

bool sorts_orders(const Problem& p) {
    // the lane CDet of a single-order batch (the split path's warp CDet and the
    // all-subsets forms have no lanes of different orders), and the queue form
    return !p.all_subsets &&
           (p.dd_mode || uses_queue_form(p) || !(p.fused_cdet && p.max_order <= kWarpCdetMaxOrder));
}

void queue_launch_shape(const Problem& p, const Scratch& w, int sm_count, int* warps_per_block, int* blocks,
                        size_t* smem) {
    const bool two_spins = !(p.same_spin[0] && p.same_spin[1]);
    const size_t ws_bytes = minors_layout(p.max_order, two_spins, true).total * sizeof(double);
    const size_t sm_bytes = 227 * 1024;  // shared memory of one SM this kernel can use (a block's limit too)
    const int sms = sm_count > 0 ? sm_count : 152;
    int per_sm = static_cast<int>(std::min<size_t>(32, sm_bytes / (ws_bytes + 16)));
    if (p.queue.warps_per_sm > 0) per_sm = std::min(per_sm, p.queue.warps_per_sm);
    if (p.queue.pair) per_sm &= ~1;
    per_sm = std::max(per_sm, p.queue.pair ? 2 : 1);
    // as few blocks per SM as blocks of at most kQueueMaxWarps allow
    int wpb = per_sm / ((per_sm + kQueueMaxWarps - 1) / kQueueMaxWarps);
    if (p.queue.pair) wpb &= ~1;
    // the pair exchange: four doubles per pair of warps
    size_t bytes = ws_bytes * wpb + (p.queue.pair ? 2 * static_cast<size_t>(wpb) * sizeof(double) : 0);
    int per_sm_blocks = std::max(1, per_sm / wpb);
    while (per_sm_blocks > 1 && per_sm_blocks * (bytes + 1024) > sm_bytes + 1024) --per_sm_blocks;
    int64_t grid = static_cast<int64_t>(sms) * per_sm_blocks;
    // the LU-fallback scratch holds ws_warps warps; no more warps than configurations need
    grid = std::min<int64_t>(grid, std::max<int64_t>(1, static_cast<int64_t>(w.ws_warps) / wpb));
    const int64_t warps_needed = p.batch * (p.queue.pair ? 2 : 1);
    grid = std::min<int64_t>(grid, std::max<int64_t>(1, (warps_needed + wpb - 1) / wpb));
    *warps_per_block = wpb;
    *blocks = static_cast<int>(grid);
    *smem = bytes;
}

cudaError_t launch_fp64_integrand(const Problem& p_in, const Scratch& w, int sm_count,
                                  cudaStream_t stream, const KernelEvents* events, bool assembly) {
    if (p_in.batch <= 0) return cudaSuccess;
    auto mark = [&](int k) {
        if (events && events->marks[k]) cudaEventRecord(events->marks[k], stream);
    };
    if (assembly) {
        mark(0);
        mark(1);
        const int64_t entries = p_in.batch * 2 * static_cast<int64_t>(p_in.max_order) * p_in.max_order;
        const unsigned grid = static_cast<unsigned>((entries + 127) / 128);
        if (p_in.reuse_mask && p_in.all_subsets) {
            // Green-pair reuse: scan of the fresh entries, copies, compacted evaluations
            // (the configurations' slot array is free in an all-subsets evaluation)
            reuse_scan<<<1, 1024, 0, stream>>>(p_in, w.slot_of, w.order_count + kReuseTotalIndex);
            green_copy_retained<<<grid, 128, 0, stream>>>(p_in, w);
            green_assembly_fp64_fresh<<<grid, 128, 0, stream>>>(p_in, w, w.slot_of, w.order_count + kReuseTotalIndex);
        } else {
            green_assembly_fp64<<<grid, 128, 0, stream>>>(p_in, w);
        }
        const cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) return err;
        mark(2);
    }
    return post_assembly(p_in, w, sm_count, stream, events);
}

cudaError_t launch_post_assembly(const Problem& p, const Scratch& w, int sm_count, cudaStream_t stream) {
    if (p.batch <= 0) return cudaSuccess;
    return post_assembly(p, w, sm_count, stream, nullptr);
}

int all_subsets_lane_form_min_batch(int sm_count) {
    // without a measurement: the lane form from one warp of configurations per SM
    return (sm_count > 0 ? sm_count : 152) * kWarp;
}

}  // namespace cdet
