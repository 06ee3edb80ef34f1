// Split-precision Green-matrix assembly on the tcgen05 tensor cores (sm_103a).
//
// The Chebyshev sum G = sum_{a,b} C[a][b] T_a(u) T_b(v) of one lookup is
// evaluated for all lookups of one coefficient block together:
//
//   W[a][l] = sum_b C[a][b] T_b(v_l)        (tensor cores, exact)
//   G_l     = sum_a T_a(u_l) W[a][l]          (integer epilogue, exact up to
//                                             final rounding)
//
// Operands are split Ozaki-style into fp16 slices of balanced 8-bit digits:
// C = 2^E sum_t q_t 2^{-8t} per block (E = the block's binary exponent, eight
// digits, |q_1| <= 256, |q_t| <= 128) and T_b(v) = sum_t' q'_t' 2^{-8t'}
// (seven digits of the Q56 fixed-point value). Every product of two digits is
// an exact integer below 2^16, and the FP32 accumulation of the products of
// one level tau = t + t' over K <= 128 stays within 2^24 for tau <= 7, so the
// accumulators of levels 2..7 in tensor memory hold exact integers. Level 8
// also takes the eighth coefficient digit, stored pre-scaled by 2^-8, and
// carries weight 2^-64; products of levels 9 and above (weight 2^-72) are
// dropped. The epilogue combines the levels in 64-bit fixed point (2^-55),
// multiplies by T_a(u) in Q62 fixed point and sums over a in 128-bit
// integers. Against an exact evaluation of the series the result is within
// 1.4e-16 of the block's largest coefficient at degree 16, 2.3e-16 at degree
// 64 and 3.8e-16 at degree 160 (the FP64 Clenshaw sum: 4e-15 to 1.2e-14):
// FP64-level accuracy without the FP64 pipe.
//
// Both bases come from the stride-2 Chebyshev recurrence
// T_{n+2} = 2 T_2 T_n - T_{n-2} in Q62 fixed point, one thread of a pair for
// the even and one for the odd degrees. To let each thread write whole
// core-matrix rows, the coefficient slices order each K step of 16 columns as
// the eight even b followed by the eight odd b; the contraction over k is
// indifferent to the order.
//
// Pipeline per evaluation: split_descriptors (one thread per vertex pair:
// branch, u, v, block ids; corner entries written directly), a counting sort
// of lookups by block (histogram, single-CTA scan, scatter), a tile list of
// up to 64 lookups of one block, and split_assembly, a persistent kernel with
// one CTA per SM that runs the tcgen05 GEMM of each tile. A-operand slices
// stream from HBM with bulk asynchronous copies (cp.async.bulk) into a
// three-stage shared-memory ring; the basis slices are generated in shared
// memory by four producer warps while a single thread issues the MMAs and
// four epilogue warps drain the previous tile.
//
// Degrees above 128 (up to 256) cut each coefficient block into sub-blocks of
// 128 rows x 128 columns (the last ones shorter: the K steps of a column
// chunk end at its last column, its rows are zero padded), which keeps every
// exact level within K <= 128. A lookup becomes one record per sub-block; the
// producers and the epilogue start the v and u recurrences at the
// sub-block's first degree, every part is left as an exact 128-bit integer on
// the block's common scale, and split_combine adds the parts and rounds once.
#include "cdet_device.cuh"
#include "cdet_kernels.cuh"

#include <cuda_fp16.h>

#include <algorithm>

namespace cdet {

namespace {

constexpr int kSlices = 7;          // slices of the basis operand
constexpr int kSlicesA = 8;         // slices of the coefficient operand (the eighth pre-scaled by 2^-8)
constexpr int kLevels = 7;          // accumulator levels tau = 2..8
constexpr int kSubK = 128;          // K columns of one sub-block: keeps every exact level below 2^24
constexpr int kTileN = 64;          // lookups per tile (MMA N)
constexpr int kRows = 128;          // MMA M (Chebyshev rows a, zero padded)
constexpr int kKStep = 16;          // MMA K (bf16)
constexpr int kSubKSteps = kSubK / kKStep;  // K steps of a full column chunk
constexpr long long kWaitCycles = 2000000000LL;  // ~1 s at 2 GHz: bound of every mbarrier wait

// bytes of one A stage: 8 slices x 128 rows x 16 k x fp16
constexpr uint32_t kAStageBytes = kSlicesA * kRows * kKStep * 2;      // 32 KiB
// bytes of the B operand of one K step: 7 slices x 64 lookups x 16 k x fp16
constexpr uint32_t kBStepBytes = kSlices * kTileN * kKStep * 2;       // 14 KiB
// Q56 basis value -> byte digits: +128 on each of the six low bytes makes
// every byte a balanced digit plus 128; +256 at bit 56 makes the top field
// (bits 48 and up) the leading digit plus 256, in [0, 512].
constexpr uint64_t kDigitBias = 0x0100808080808080ull;

// ----------------------------------------------------------- PTX helpers --
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor, K-major, no swizzle: core matrices of
// 8 rows x 16 bytes; lbo = byte stride between core matrices along K, sbo =
// byte stride between 8-row groups.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
    d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
    d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
    d |= static_cast<uint64_t>(1) << 46;
    return d;
}

// kind::f16 instruction descriptor: f16 x f16 -> f32, K-major A and B.
__host__ __device__ constexpr uint32_t mma_idesc(int m, int n) {
    return (1u << 4) | (static_cast<uint32_t>(n >> 3) << 17) | (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes));
}

// Wait for the phase with the given parity, for at most kWaitCycles SM
// clocks; returns false on timeout (the caller records an error and stops).
// Each try_wait may suspend the thread until the phase completes (at most
// kSuspendNs), so a waiting warp takes no issue slots from the warps that
// share its scheduler.
constexpr uint32_t kSuspendNs = 200000;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done = 0;
    const long long start = clock64();
    while (true) {
        asm volatile(
            "{.reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3; selp.u32 %0, 1, 0, p;}"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity), "r"(kSuspendNs)
            : "memory");
        if (done) return true;
        if (clock64() - start > kWaitCycles) return false;
    }
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void mma_f16(uint32_t tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{.reg .pred p; setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;}\n" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
        smem_addr(bar)));
}

// ------------------------------------------------------ fixed-point helpers --
// round(x * 2^frac) as int64 for |x| <= 1, by integer operations on the bits.
__device__ __forceinline__ int64_t fixed_from_double(double x, int frac) {
    const uint64_t bits = static_cast<uint64_t>(__double_as_longlong(x));
    const int e = static_cast<int>((bits >> 52) & 0x7FF);
    if (e == 0) return 0;
    const int64_t mant = static_cast<int64_t>((bits & ((uint64_t{1} << 52) - 1)) | (uint64_t{1} << 52));
    const int shift = e - 1075 + frac;
    int64_t v;
    if (shift >= 0) v = mant << shift;
    else if (shift > -60) v = (mant + (int64_t{1} << (-shift - 1))) >> (-shift);
    else v = 0;
    return (bits >> 63) ? -v : v;
}

// (hi:lo) * 2^scale_exp as a double, rounded to nearest even, with integer
// operations only (the FP64 pipe is narrow). Results outside the normal
// range take the FP64 route.
__device__ __forceinline__ double int128_to_double(int64_t hi, uint64_t lo, int scale_exp) {
    const bool neg = hi < 0;
    uint64_t mhi = static_cast<uint64_t>(hi), mlo = lo;
    if (neg) {
        mlo = ~mlo + 1;
        mhi = ~mhi + (mlo == 0 ? 1 : 0);
    }
    if ((mhi | mlo) == 0) return 0.0;
    const int lz = mhi ? __clzll(static_cast<long long>(mhi)) : 64 + __clzll(static_cast<long long>(mlo));
    // normalise so that the leading one is bit 127
    uint64_t nhi, nlo;
    if (lz >= 64) {
        nhi = mlo << (lz - 64);
        nlo = 0;
    } else if (lz > 0) {
        nhi = (mhi << lz) | (mlo >> (64 - lz));
        nlo = mlo << lz;
    } else {
        nhi = mhi;
        nlo = mlo;
    }
    uint64_t mant = nhi >> 11;  // 53 bits
    const bool round_bit = (nhi >> 10) & 1;
    const bool sticky = ((nhi & 0x3FFu) | nlo) != 0;
    int msb = 127 - lz;
    if (round_bit && (sticky || (mant & 1))) {
        ++mant;
        if (mant >> 53) {
            mant >>= 1;
            ++msb;
        }
    }
    const int field = msb + scale_exp + 1023;
    if (field <= 0 || field >= 2047) {
        const double m = static_cast<double>(mant);  // exact, 53 bits
        return ldexp(neg ? -m : m, msb - 52 + scale_exp);
    }
    const uint64_t bits = (neg ? (uint64_t{1} << 63) : 0) | (static_cast<uint64_t>(field) << 52) |
                          (mant & ((uint64_t{1} << 52) - 1));
    return __longlong_as_double(static_cast<long long>(bits));
}

// One step of the Chebyshev recurrence T_{k+1} = 2 u T_k - T_{k-1} in Q62
// fixed point (u, T in [-1, 1] scaled by 2^62). The 128-bit product is
// rounded to Q62; the wrap-around 64-bit arithmetic is exact because the
// result lies in [-1, 1]. The rounding error per step is 2^-63 and grows at
// most like k^2 (about 2^-50 at degree 128), 2^11 below the FP64 recurrence.
__device__ __forceinline__ int64_t cheb_step_q62(int64_t ufix, int64_t t, int64_t tprev) {
    const uint64_t lo = static_cast<uint64_t>(ufix) * static_cast<uint64_t>(t);
    uint64_t hi = static_cast<uint64_t>(__mul64hi(ufix, t));
    const uint64_t lo2 = lo + (uint64_t{1} << 60);
    hi += lo2 < lo ? 1u : 0u;
    const uint64_t twice = (hi << 3) | (lo2 >> 61);  // round(2 u t) in Q62, modulo 2^64
    return static_cast<int64_t>(twice - static_cast<uint64_t>(tprev));
}

// Two fp16 digits (the same slice of two consecutive k) from the biased
// basis values ya, yb. Slice 1 is the top field (bits 48..57, leading digit
// + 256); slices 2..7 are bytes 5..0 (digit + 128). A field f < 1024 placed
// in the mantissa of 1024 is the fp16 number 1024 + f; one packed
// subtraction removes 1024 and the bias exactly.
__device__ __forceinline__ uint32_t digit_pair(uint64_t ya, uint64_t yb, int slice) {
    uint32_t r;
    __half2 bias;
    if (slice == 1) {
        r = __byte_perm(static_cast<uint32_t>(ya >> 32), static_cast<uint32_t>(yb >> 32), 0x7632) | 0x64006400u;
        bias = __halves2half2(__ushort_as_half(0x6500), __ushort_as_half(0x6500));  // 1280
    } else {
        const int byte = 7 - slice;  // 5..0
        const uint32_t wa = byte >= 4 ? static_cast<uint32_t>(ya >> 32) : static_cast<uint32_t>(ya);
        const uint32_t wb = byte >= 4 ? static_cast<uint32_t>(yb >> 32) : static_cast<uint32_t>(yb);
        const uint32_t bi = static_cast<uint32_t>(byte & 3);
        r = (__byte_perm(wa, wb, bi | (bi << 4) | ((bi + 4) << 8) | ((bi + 4) << 12)) & 0x00FF00FFu) | 0x64006400u;
        bias = __halves2half2(__ushort_as_half(0x6480), __ushort_as_half(0x6480));  // 1152
    }
    __half2 h = *reinterpret_cast<__half2*>(&r);
    h = __hsub2(h, bias);
    return *reinterpret_cast<uint32_t*>(&h);
}

// Offset (in 16-bit elements) of element (row, k) inside one K-major
// no-swizzle operand of `rows` rows and 16 k: [row group][k chunk][8][8].
__device__ __forceinline__ int core_offset(int row, int k) {
    return (row >> 3) * 128 + (k >> 3) * 64 + (row & 7) * 8 + (k & 7);
}

// ---------------------------------------------------------- table slicing --
// One sub-block (rows 128 rb.., columns 128 kc..) of a block of nu x nv FP64
// coefficients -> kSlicesA fp16 slices laid out as [kstep][slice][core layout
// of 128 rows x 16 k], and (by sub-block 0) the block exponent, taken over the
// whole block so that all its sub-blocks share one scale. Degrees up to 128
// make one sub-block per block; up to 256, two per dimension.
// Within K step ks, position k holds column b = 16 ks + 2k (k < 8) or
// 16 ks + 2(k - 8) + 1 (k >= 8), the order in which the basis threads produce
// T_b(v). Slices 1..7 are integers q_t (weight 2^-8t); slice 8 is stored as
// q_8 * 2^-8 (exact in fp16) so that its one product, with the first basis
// slice, accumulates at level 8 with the right weight. Eight digits leave a
// truncation of 2^-65 of the block scale per coefficient.
__host__ __device__ __forceinline__ int row_ksteps(int nkc, int ksteps_last) {
    return (nkc - 1) * kSubKSteps + ksteps_last;
}

__global__ void __launch_bounds__(256) slice_blocks(const double* __restrict__ coeffs, int nu, int nv,
                                                    int nrb, int nkc, int ksteps_last,
                                                    uint16_t* __restrict__ out, int32_t* __restrict__ exponents) {
    const int nsub = nrb * nkc;
    const int64_t block = blockIdx.x / nsub;
    const int sub = static_cast<int>(blockIdx.x - block * nsub);
    const int rb = sub / nkc, kc = sub - (sub / nkc) * nkc;
    const int row0 = rb * kRows, col0 = kc * kSubK;
    const int ksteps = kc == nkc - 1 ? ksteps_last : kSubKSteps;
    const int rk = row_ksteps(nkc, ksteps_last);
    const double* c = coeffs + block * static_cast<int64_t>(nu) * nv;
    __shared__ double red[256];
    double m = 0.0;
    for (int i = threadIdx.x; i < nu * nv; i += blockDim.x) m = fmax(m, fabs(c[i]));
    red[threadIdx.x] = m;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    int e = 0;
    if (red[0] > 0.0) frexp(red[0], &e);  // max < 2^e
    if (threadIdx.x == 0 && sub == 0) exponents[block] = e;
    uint16_t* dst = out + ((block * nrb + rb) * rk + static_cast<int64_t>(kc) * kSubKSteps) * (kAStageBytes / 2);
    const int total = kRows * ksteps * kKStep;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
        const int a = i / (ksteps * kKStep);
        const int b = i - a * (ksteps * kKStep);
        const int ag = row0 + a, bg = col0 + b;
        double r = (ag < nu && bg < nv) ? ldexp(c[ag * nv + bg], -e) : 0.0;  // |r| < 1
        const int ks = b / kKStep, bb = b - ks * kKStep;
        const int k = (bb & 1) * 8 + (bb >> 1);
        uint16_t* base = dst + static_cast<int64_t>(ks) * kSlicesA * kRows * kKStep + core_offset(a, k);
        for (int t = 0; t < kSlicesA; ++t) {
            // exact: r * 256 has the same significand, and subtracting the
            // nearest integer leaves the (representable) remainder
            const double scaled = r * 256.0;
            const double q = rint(scaled);
            r = scaled - q;
            const float stored = t < kSlicesA - 1 ? static_cast<float>(q) : static_cast<float>(q) * 0.00390625f;
            base[t * kRows * kKStep] = __half_as_ushort(__float2half_rn(stored));
        }
    }
}

// ------------------------------------------------------------ descriptors --
struct SplitRecordArrays {
    uint32_t* key;    // block id, or kNoKey
    double* u;
    double* v;
    uint64_t* info;   // c | set<<32 | spinmask<<33 | i<<35 | j<<40 | n<<45
};
constexpr uint32_t kNoKey = 0xFFFFFFFFu;

__device__ __forceinline__ uint64_t pack_info(int64_t c, int set, int spins, int i, int j, int n) {
    return static_cast<uint64_t>(c) | (static_cast<uint64_t>(set) << 32) |
           (static_cast<uint64_t>(spins) << 33) | (static_cast<uint64_t>(i) << 35) |
           (static_cast<uint64_t>(j) << 40) | (static_cast<uint64_t>(n) << 45);
}

__device__ __forceinline__ int coordinate_index_s(double scaled, int extent, bool& bad) {
    if (!(scaled > -2147483648.0 && scaled < 2147483648.0)) {
        bad = true;
        return 0;
    }
    int index = static_cast<int>(floor(scaled));
    if (index < 0) index = 0;
    if (index >= extent) index = extent - 1;
    return index;
}

__device__ __forceinline__ double clamp_unit_s(double value) {
    if (value < -1.0) return -1.0;
    if (value > 1.0) return 1.0;
    return value;
}

// Records per vertex pair: one per distinct up/down table of each set.
__host__ __device__ __forceinline__ int records_per_pair(const SplitPlan& plan) {
    return plan.records_per_set[0] + plan.records_per_set[1];
}

// One thread per (configuration, i, j): branch and (u, v) are shared by both
// table sets; the corner path is evaluated here, every other lookup becomes
// one record per sub-block of its coefficient block, keyed by the sub-block.
// Record slots are fixed: ((c * nmax^2 + pair) * records_per_pair + record)
// * nsub + sub, the set's records after those of the sets before it.
__global__ void __launch_bounds__(128) split_descriptors(const __grid_constant__ Problem p,
                                                         const __grid_constant__ Scratch w,
                                                         const __grid_constant__ SplitPlan plan,
                                                         SplitRecordArrays rec, uint32_t* counts) {
    const int nmax = p.max_order;
    const int64_t per_c = static_cast<int64_t>(nmax) * nmax;
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= p.batch * per_c) return;
    const int64_t c = idx / per_c;
    const int pair = static_cast<int>(idx - c * per_c);
    const int i = pair / nmax, j = pair - (pair / nmax) * nmax;
    const int nsub = plan.nrb * plan.nkc;
    const int rpp = records_per_pair(plan);
    const int64_t slot0 = idx * rpp * nsub;
    for (int k = 0; k < rpp * nsub; ++k) rec.key[slot0 + k] = kNoKey;
    const int n = p.all_subsets ? nmax : __ldg(p.orders + c);
    if (n < 1 || n > nmax) {
        if (pair == 0) atomicOr(p.status + c, kStatusBadInput);
        return;
    }
    if (i >= n || j >= n) return;
    const Scalars& s = p.s;
    const double* vb = p.vertices + c * static_cast<int64_t>(nmax) * 4;
    bool bad = false;
    const double tui = __ldg(vb + 4 * i), tuj = __ldg(vb + 4 * j);
    if (!isfinite(tui) || !isfinite(tuj)) bad = true;
    const double taui = dmul(s.beta, tui), tauj = dmul(s.beta, tuj);
    const int xi = coordinate_index_s(dmul(static_cast<double>(s.n1), __ldg(vb + 4 * i + 1)), s.n1, bad);
    const int yi = coordinate_index_s(dmul(static_cast<double>(s.n2), __ldg(vb + 4 * i + 2)), s.n2, bad);
    const int xj = coordinate_index_s(dmul(static_cast<double>(s.n1), __ldg(vb + 4 * j + 1)), s.n1, bad);
    const int yj = coordinate_index_s(dmul(static_cast<double>(s.n2), __ldg(vb + 4 * j + 2)), s.n2, bad);
    const int ri = coordinate_index_s(dmul(2.0, __ldg(vb + 4 * i + 3)), 2, bad);
    const int rj = coordinate_index_s(dmul(2.0, __ldg(vb + 4 * j + 3)), 2, bad);
    if (bad) {
        atomicOr(p.status + c, kStatusBadInput);
        return;
    }
    const bool upper = (i != j) && (tui > tuj);
    const double t_outer = upper ? taui : tauj;
    const double t_inner = upper ? tauj : taui;
    const bool corner = t_outer < s.branch_eps;
    double u = 0.0, v = 0.0;
    if (!corner) {
        u = clamp_unit_s(dsub(ddiv(dmul(2.0, t_outer), s.beta), 1.0));
        v = clamp_unit_s(dsub(ddiv(dmul(2.0, t_inner), t_outer), 1.0));
    }
    const uint64_t site_part =
        ((static_cast<uint64_t>(xi) * s.n2 + yi) * s.n1 + xj) * s.n2 + yj;
    const uint64_t sites2 = static_cast<uint64_t>(s.n1) * s.n2 * s.n1 * s.n2;
    for (int set = 0; set < 2; ++set) {
        const uint64_t sitepair =
            set == 0 ? (static_cast<uint64_t>(ri) * 2 + rj) * sites2 + site_part : site_part;
        const int64_t mslot = (c * 2 + set) * 2;
        if (corner) {
            const TableDev& tu = p.up[set];
            const TableDev& td = p.down[set];
            double up = __ldg((upper ? tu.upper_corners : tu.lower_corners) + sitepair);
            double down = p.same_spin[set] ? up
                                           : __ldg((upper ? td.upper_corners : td.lower_corners) + sitepair);
            if (i == j) {
                up = dadd(up, s.diag_up_shift);
                down = dadd(down, s.diag_down_shift);
                w.diag[mslot * nmax + i] = up;
                w.diag[(mslot + 1) * nmax + i] = down;
            }
            w.green[mslot * per_c + i * n + j] = dmul(up, s.scale);
            w.green[(mslot + 1) * per_c + i * n + j] = dmul(down, s.scale);
            continue;
        }
        for (int r = 0; r < plan.records_per_set[set]; ++r) {
            const int seg = plan.segment_of[set][r][upper ? 0 : 1];
            const uint64_t info = pack_info(c, set, plan.spin_mask[set][r], i, j, n);
            for (int sub = 0; sub < nsub; ++sub) {
                const uint32_t key = plan.segment_base[seg] + static_cast<uint32_t>(sitepair * nsub + sub);
                const int64_t slot = slot0 + ((set ? plan.records_per_set[0] : 0) + r) * nsub + sub;
                rec.key[slot] = key;
                rec.u[slot] = u;
                rec.v[slot] = v;
                rec.info[slot] = info;
                atomicAdd(counts + key, 1u);
            }
        }
    }
}

// Exclusive scan of block counts (offsets) and of their 64-lookup tile counts
// (tile offsets); one CTA of 1024 threads. totals[0] = lookups, totals[1] = tiles.
__global__ void __launch_bounds__(1024) split_scan(const uint32_t* __restrict__ counts, uint32_t nblocks,
                                                   uint32_t* __restrict__ offsets,
                                                   uint32_t* __restrict__ tile_offsets,
                                                   uint32_t* __restrict__ cursors,
                                                   uint32_t* __restrict__ totals) {
    __shared__ uint32_t s_sum[1024], s_tiles[1024];
    const uint32_t per = (nblocks + 1023) / 1024;
    const uint32_t begin = threadIdx.x * per;
    const uint32_t end = min(nblocks, begin + per);
    uint32_t sum = 0, tiles = 0;
    for (uint32_t b = begin; b < end; ++b) {
        sum += counts[b];
        tiles += (counts[b] + kTileN - 1) / kTileN;
    }
    s_sum[threadIdx.x] = sum;
    s_tiles[threadIdx.x] = tiles;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        uint32_t a = 0, t = 0;
        if (threadIdx.x >= static_cast<unsigned>(off)) {
            a = s_sum[threadIdx.x - off];
            t = s_tiles[threadIdx.x - off];
        }
        __syncthreads();
        s_sum[threadIdx.x] += a;
        s_tiles[threadIdx.x] += t;
        __syncthreads();
    }
    uint32_t run = s_sum[threadIdx.x] - sum, trun = s_tiles[threadIdx.x] - tiles;
    for (uint32_t b = begin; b < end; ++b) {
        offsets[b] = run;
        tile_offsets[b] = trun;
        cursors[b] = 0;
        run += counts[b];
        trun += (counts[b] + kTileN - 1) / kTileN;
    }
    if (threadIdx.x == 1023) {
        totals[0] = s_sum[1023];
        totals[1] = s_tiles[1023];
    }
}

struct SplitTile {
    uint32_t block, start, count, pad;
};

// Scatter records into block order and emit the tile list.
__global__ void __launch_bounds__(256) split_scatter(const SplitRecordArrays rec, int64_t nrec,
                                                     const uint32_t* __restrict__ offsets,
                                                     uint32_t* __restrict__ cursors,
                                                     SplitRecordArrays sorted) {
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= nrec) return;
    const uint32_t key = rec.key[idx];
    if (key == kNoKey) return;
    const uint32_t pos = offsets[key] + atomicAdd(cursors + key, 1u);
    sorted.u[pos] = rec.u[idx];
    sorted.v[pos] = rec.v[idx];
    sorted.info[pos] = rec.info[idx];
}

__global__ void __launch_bounds__(256) split_tiles(const uint32_t* __restrict__ counts, uint32_t nblocks,
                                                   const uint32_t* __restrict__ offsets,
                                                   const uint32_t* __restrict__ tile_offsets,
                                                   SplitTile* __restrict__ tiles) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblocks) return;
    const uint32_t n = counts[b];
    uint32_t t = tile_offsets[b];
    for (uint32_t s = 0; s < n; s += kTileN, ++t) tiles[t] = SplitTile{b, offsets[b] + s, min(kTileN * 1u, n - s), 0};
}

// ------------------------------------------------------------- assembly --
// Warp-specialised persistent kernel, one CTA of 10 warps per SM:
//   warps 0-3  basis producers: the eight bf16 slices of T_b(v) for each
//              K step of a tile, into a two-stage ring (16-byte stores of
//              whole core-matrix rows, conflict-free);
//   warps 4-7  epilogue: the Q62 u-basis of the tile (while the MMAs run),
//              then the TMEM levels row by row (warp w reads lanes
//              32(w-4)..), combined in fixed point and summed over rows
//              through a shared-memory stage, and the Green entries written;
//   warp 8     one thread streams the coefficient slices of every K step
//              into a three-stage ring with cp.async.bulk;
//   warp 9     one thread issues the 37 tcgen05.mma of each K step and
//              owns the 512 TMEM columns (eight levels x 64 lookups).
// The accumulators are single-buffered: the MMAs of a tile start when the
// epilogue has released the previous tile's TMEM.
constexpr int kAStages = 3;
constexpr int kBStages = 3;
constexpr int kMetaBufs = 3;
constexpr int kProducerWarps = 4;
constexpr int kEpilogueGroups = 2;                    // each reads all 128 TMEM lanes for half the lookups
constexpr int kEpilogueWarps = 4 * kEpilogueGroups;
constexpr int kGroupLookups = kTileN / kEpilogueGroups;
constexpr int kWarpCopy = kProducerWarps + kEpilogueWarps;
constexpr int kWarpMma = kWarpCopy + 1;
constexpr int kAssemblyThreads = (kWarpMma + 1) * 32;
constexpr int kRedChunk = 8;  // lookups per epilogue reduction chunk
constexpr uint32_t kEpiBarrier = 1;       // named barrier of all epilogue warps (votes)
constexpr uint32_t kGroupBarrier0 = 2;    // named barriers of the epilogue groups: 2, 3

struct TileMeta {
    double u[kTileN];
    uint64_t info[kTileN];
    uint32_t count;
    int32_t exponent;
    int32_t sub;
    uint32_t pad;
};

struct SplitShared {
    alignas(1024) uint16_t a_ring[kAStages][kAStageBytes / 2];  // 3 x 32 KiB
    alignas(1024) uint16_t b_ring[kBStages][kBStepBytes / 2];   // 3 x 14 KiB
    alignas(16) int64_t ubasis[kTileN * kRows];                 // 64 KiB, [l][a ^ (l & 31)]
    alignas(16) int64_t red[kEpilogueGroups][kRedChunk * kRows];  // 2 x 8 KiB, [j][row]
    alignas(16) int64_t sums[kTileN][2];                        // 1 KiB, (lo, hi) per lookup
    TileMeta meta[kMetaBufs];
    uint64_t a_full[kAStages], a_empty[kAStages];
    uint64_t b_full[kBStages], b_empty[kBStages];
    uint64_t meta_full[kMetaBufs], meta_empty[kMetaBufs];
    uint64_t acc_full;
    uint64_t acc_empty[kLevels];  // per accumulator level: drained, the next tile may write it
    uint64_t drain;  // last commit of the MMA thread, waited on before dealloc
    uint32_t tmem_base;
    uint32_t error;
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// barrier of one epilogue group (128 threads)
__device__ __forceinline__ void group_sync(int group) {
    asm volatile("bar.sync %0, %1;" ::"r"(kGroupBarrier0 + group), "n"(128) : "memory");
}

// Barrier of all epilogue warps that also ORs a predicate over them: every
// epilogue thread gets the same answer, so they leave the tile loop together
// and none is left waiting at a named barrier.
__device__ __forceinline__ bool epilogue_any(bool pred) {
    uint32_t r;
    asm volatile(
        "{.reg .pred p, q; setp.ne.u32 p, %1, 0; bar.red.or.pred q, %2, %3, p; selp.u32 %0, 1, 0, q;}"
        : "=r"(r)
        : "r"(static_cast<uint32_t>(pred)), "n"(kEpiBarrier), "n"(kEpilogueWarps * 32)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ bool failed(const SplitShared& sh) {
    return *static_cast<const volatile uint32_t*>(&sh.error) != 0;
}

// Where the lookups of sort key `key` (one sub-block of one coefficient block)
// find their coefficient slices, the block exponent, and the sub-block's
// place: sub = rb * nkc + kc covers rows 128 rb.. and columns 128 kc.. in
// `ksteps` K steps.
struct TileSource {
    const uint16_t* a;
    int exponent, sub, rb, kc, ksteps;
};
template <bool Chunked>
__device__ __forceinline__ TileSource tile_source(const SplitPlan& plan, uint32_t key) {
    int seg = 0;
    while (seg + 1 < plan.segments && key >= plan.segment_base[seg + 1]) ++seg;
    const uint32_t local = key - plan.segment_base[seg];
    if constexpr (!Chunked) {  // one sub-block per block
        TileSource t;
        t.sub = t.rb = t.kc = 0;
        t.ksteps = plan.ksteps_last;
        t.a = plan.slices[seg] + static_cast<int64_t>(local) * plan.ksteps_last * (kAStageBytes / 2);
        t.exponent = plan.exponents[seg][local];
        return t;
    }
    const uint32_t nsub = static_cast<uint32_t>(plan.nrb * plan.nkc);
    const uint32_t block = local / nsub;
    TileSource t;
    t.sub = static_cast<int>(local - block * nsub);
    t.rb = t.sub / plan.nkc;
    t.kc = t.sub - t.rb * plan.nkc;
    t.ksteps = t.kc == plan.nkc - 1 ? plan.ksteps_last : kSubKSteps;
    const int rk = row_ksteps(plan.nkc, plan.ksteps_last);
    t.a = plan.slices[seg] +
          ((static_cast<int64_t>(block) * plan.nrb + t.rb) * rk + static_cast<int64_t>(t.kc) * kSubKSteps) *
              (kAStageBytes / 2);
    t.exponent = plan.exponents[seg][block];
    return t;
}

// Column chunk of sort key `key` and its K steps, without the slice address
// (constant when the columns make one chunk).
__device__ __forceinline__ int tile_kc(const SplitPlan& plan, uint32_t key) {
    if (plan.nkc == 1) return 0;
    int seg = 0;
    while (seg + 1 < plan.segments && key >= plan.segment_base[seg + 1]) ++seg;
    const uint32_t nsub = static_cast<uint32_t>(plan.nrb * plan.nkc);
    return static_cast<int>(((key - plan.segment_base[seg]) % nsub) % static_cast<uint32_t>(plan.nkc));
}
__device__ __forceinline__ int chunk_ksteps(const SplitPlan& plan, int kc) {
    return kc == plan.nkc - 1 ? plan.ksteps_last : kSubKSteps;
}

// The Green entries of one lookup's value (both spins of a shared record),
// with the diagonal shift and the scale, as the FP64 assembly writes them.
__device__ __forceinline__ void store_green(const Problem& p, const Scratch& w, uint64_t info, double value) {
    const int nmax = p.max_order;
    const int64_t per_c = static_cast<int64_t>(nmax) * nmax;
    const int64_t c = static_cast<int64_t>(info & 0xFFFFFFFFu);
    const int set = static_cast<int>((info >> 32) & 1);
    const int spins = static_cast<int>((info >> 33) & 3);
    const int i = static_cast<int>((info >> 35) & 31);
    const int jj = static_cast<int>((info >> 40) & 31);
    const int n = static_cast<int>((info >> 45) & 31);
    const int64_t mslot = (c * 2 + set) * 2;
    for (int spin = 0; spin < 2; ++spin) {
        if (!(spins & (1 << spin))) continue;
        double g = value;
        if (i == jj) {
            g = dadd(g, spin == 0 ? p.s.diag_up_shift : p.s.diag_down_shift);
            w.diag[(mslot + spin) * nmax + i] = g;
        }
        w.green[(mslot + spin) * per_c + i * n + jj] = dmul(g, p.s.scale);
    }
}

// Record slot of a lookup's sub-block part (the slot its descriptor filled).
__device__ __forceinline__ int64_t part_slot(uint64_t info, const SplitPlan& plan, int nmax, int sub) {
    const int64_t c = static_cast<int64_t>(info & 0xFFFFFFFFu);
    const int set = static_cast<int>((info >> 32) & 1);
    const int spins = static_cast<int>((info >> 33) & 3);
    const int i = static_cast<int>((info >> 35) & 31);
    const int jj = static_cast<int>((info >> 40) & 31);
    const int record = spins == 2 ? 1 : 0;  // the spin-down record of a set with two tables
    const int64_t nsub = plan.nrb * plan.nkc;
    return (((c * nmax + i) * nmax + jj) * records_per_pair(plan) + (set ? plan.records_per_set[0] : 0) + record) *
               nsub + sub;
}

// T_parity, T_{parity+2}, T_{parity+4}, ... of x in Q62 fixed point, by the
// stride-2 recurrence T_{n+2} = 2 T_2(x) T_n - T_{n-2}, started from
// (T_{-2}, T_0) = (T_2, 1) or (T_{-1}, T_1) = (x, x). The recurrence in
// w = T_2(x) has half the steps of the stride-1 one and its rounding error
// grows like the square of the step count.
struct ChebStride2;
// T_r, T_{r+4}, T_{r+8}, ... (r = 0..3) of x in Q62 fixed point, by
// T_{n+4} = 2 T_4(x) T_n - T_{n-4}, started from (T_{r-4}, T_r) = (T_{4-r}, T_r).
struct ChebStride4 {
    int64_t w, prev, cur;
    __device__ __forceinline__ void init(int64_t xfix, int r) {
        const int64_t one = int64_t{1} << 62;
        const int64_t t2 = cheb_step_q62(xfix, xfix, one);
        const int64_t t3 = cheb_step_q62(xfix, t2, xfix);
        const int64_t t4 = cheb_step_q62(xfix, t3, t2);
        w = t4;
        cur = r == 0 ? one : r == 1 ? xfix : r == 2 ? t2 : t3;
        prev = r == 0 ? t4 : r == 1 ? t3 : r == 2 ? t2 : xfix;
    }
    __device__ __forceinline__ int64_t next() {
        const int64_t t = cur;
        cur = cheb_step_q62(w, cur, prev);
        prev = t;
        return t;
    }
};

struct ChebStride2 {
    int64_t w, prev, cur;
    __device__ __forceinline__ void init(int64_t xfix, int parity) {
        w = cheb_step_q62(xfix, xfix, int64_t{1} << 62);  // 2 x^2 - 1
        prev = parity ? xfix : w;
        cur = parity ? xfix : (int64_t{1} << 62);
    }
    __device__ __forceinline__ int64_t next() {
        const int64_t t = cur;
        cur = cheb_step_q62(w, cur, prev);
        prev = t;
        return t;
    }
};

template <bool Chunked>
__global__ void __launch_bounds__(kAssemblyThreads, 1) split_assembly(const __grid_constant__ Problem p,
                                                                      const __grid_constant__ Scratch w,
                                                                      const __grid_constant__ SplitPlan plan,
                                                                      const SplitRecordArrays sorted,
                                                                      const SplitTile* __restrict__ tiles,
                                                                      const uint32_t* __restrict__ totals,
                                                                      int64_t* __restrict__ parts,
                                                                      int32_t* __restrict__ error_flag,
                                                                      unsigned long long* __restrict__ counters) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    SplitShared& sh = *reinterpret_cast<SplitShared*>(smem_raw);
    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;
    const uint32_t ntiles = totals[1];
    // each CTA takes a contiguous range of the block-sorted tile list, so the
    // later tiles of a coefficient block find its slices in L2
    const uint32_t tile_begin =
        static_cast<uint32_t>((static_cast<uint64_t>(ntiles) * blockIdx.x) / gridDim.x);
    const uint32_t tile_end =
        static_cast<uint32_t>((static_cast<uint64_t>(ntiles) * (blockIdx.x + 1)) / gridDim.x);

    if (tid == 0) {
        for (int i = 0; i < kAStages; ++i) {
            mbar_init(&sh.a_full[i], 1);
            mbar_init(&sh.a_empty[i], 1);
        }
        for (int i = 0; i < kBStages; ++i) {
            mbar_init(&sh.b_full[i], kProducerWarps * 32);
            mbar_init(&sh.b_empty[i], 1);
        }
        for (int i = 0; i < kMetaBufs; ++i) {
            mbar_init(&sh.meta_full[i], kProducerWarps * 32);
            mbar_init(&sh.meta_empty[i], kEpilogueWarps * 32);
        }
        mbar_init(&sh.acc_full, 1);
        for (int i = 0; i < kLevels; ++i) mbar_init(&sh.acc_empty[i], kEpilogueWarps * 32);
        mbar_init(&sh.drain, 1);
        sh.error = 0;
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == kWarpMma) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
            smem_addr(&sh.tmem_base)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = sh.tmem_base;

    if (warp < kProducerWarps) {
        // ---------------------------------------------- basis producers --
        // lanes 0-15 of a warp: lookups 16w..16w+15, even degrees; lanes
        // 16-31: the same lookups, odd degrees
        const int l = warp * 16 + (lane & 15);  // lookup of this thread
        const int h = lane >> 4;                // parity of its degrees = which 8 of the 16 k
        uint32_t b_cnt = 0, tile_cnt = 0;
        for (uint32_t tile = tile_begin; tile < tile_end && !failed(sh); ++tile, ++tile_cnt) {
            const SplitTile tl = tiles[tile];
            const int mb = static_cast<int>(tile_cnt % kMetaBufs);
            if (tile_cnt >= kMetaBufs && !mbar_wait(&sh.meta_empty[mb], ((tile_cnt / kMetaBufs) - 1) & 1)) {
                sh.error = 1;
                break;
            }
            const bool live = static_cast<uint32_t>(l) < tl.count;
            const double v = live ? sorted.v[tl.start + l] : 0.0;
            if (h == 0) {
                sh.meta[mb].u[l] = live ? sorted.u[tl.start + l] : 0.0;
                sh.meta[mb].info[l] = live ? sorted.info[tl.start + l] : ~uint64_t{0};
            }
            if (tid == 0) {
                const TileSource src = tile_source<Chunked>(plan, tl.block);
                sh.meta[mb].count = tl.count;
                sh.meta[mb].exponent = src.exponent;
                sh.meta[mb].sub = src.sub;
            }
            mbar_arrive(&sh.meta_full[mb]);
            int ksteps = plan.ksteps_last, b0 = 0;
            ChebStride2 cheb;
            cheb.init(fixed_from_double(v, 62), h);
            if constexpr (Chunked) {
                const int kc = tile_kc(plan, tl.block);
                ksteps = chunk_ksteps(plan, kc);
                b0 = kc * kSubK;
                for (int k = 0; k < kc * kSubK / 2; ++k) cheb.next();  // to degree 128 kc + h
            }
            for (int ks = 0; ks < ksteps; ++ks, ++b_cnt) {
                const int sb = static_cast<int>(b_cnt % kBStages);
                if (b_cnt >= kBStages && !mbar_wait(&sh.b_empty[sb], ((b_cnt / kBStages) - 1) & 1)) {
                    sh.error = 1;
                    break;
                }
                // k = 8h + j holds b = 16 ks + 2j + h
                uint64_t y[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int b = b0 + ks * kKStep + 2 * j + h;
                    const int64_t tb = cheb.next();
                    const int64_t x = b < p.s.nv ? (tb + 32) >> 6 : 0;  // Q56
                    y[j] = static_cast<uint64_t>(x) + kDigitBias;
                }
                uint16_t* base = sh.b_ring[sb] + core_offset(l, 8 * h);
#pragma unroll
                for (int t = 1; t <= kSlices; ++t) {
                    const uint32_t addr = smem_addr(base + (t - 1) * kTileN * kKStep);
                    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(digit_pair(y[0], y[1], t)),
                                 "r"(digit_pair(y[2], y[3], t)), "r"(digit_pair(y[4], y[5], t)),
                                 "r"(digit_pair(y[6], y[7], t))
                                 : "memory");
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(&sh.b_full[sb]);
            }
        }
    } else if (warp < kProducerWarps + kEpilogueWarps) {
        // ------------------------------------------------------ epilogue --
        const int e = tid - kProducerWarps * 32;       // 0..255
        const int group = e >> 7;                      // lookups [32 group, 32 group + 32)
        const int row = e & (kRows - 1);               // TMEM lane = Chebyshev row a
        const uint32_t lane_base = tmem + (static_cast<uint32_t>((warp & 3) * 32) << 16);
        const int nu = p.s.nu;
        const int nmax = p.max_order;
        int64_t* red = sh.red[group];
        uint32_t tile_cnt = 0;
        for (uint32_t tile = tile_begin; tile < tile_end; ++tile, ++tile_cnt) {
            const int mb = static_cast<int>(tile_cnt % kMetaBufs);
            const bool meta_ok = mbar_wait(&sh.meta_full[mb], (tile_cnt / kMetaBufs) & 1);
            // (also: every epilogue thread is done with the previous tile's u basis)
            if (epilogue_any(!meta_ok || failed(sh))) {
                sh.error = 1;
                break;
            }
            const TileMeta& meta = sh.meta[mb];
            // u basis of the tile, four threads per lookup (degrees r mod 4);
            // each half-warp holds 16 lookups of one residue, so its stores
            // hit 16 distinct bank pairs
            {
                const int we = e >> 5;
                const int l = 16 * (we & 3) + (lane & 15), r = 2 * (we >> 2) + (lane >> 4);
                ChebStride4 cheb;
                cheb.init(fixed_from_double(meta.u[l], 62), r);
                int a0 = 0;  // first row of the sub-block
                if constexpr (Chunked) {
                    a0 = (meta.sub / plan.nkc) * kRows;
                    for (int k = 0; k < a0 / 4; ++k) cheb.next();  // to degree a0 + r
                }
                for (int a = r; a < kRows; a += 4) {
                    const int64_t ta = cheb.next();
                    sh.ubasis[l * kRows + (a ^ (l & 31))] = a0 + a < nu ? ta : 0;
                }
            }
            const bool acc_ok = mbar_wait(&sh.acc_full, tile_cnt & 1);
            if (epilogue_any(!acc_ok)) {  // also orders the u-basis stores before their reads
                sh.error = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t count = meta.count;
            const int exponent = meta.exponent;
            // Drain: every accumulator of this thread's row and the group's 32
            // lookups into 64-bit fixed point, W * 2^55 = sum_tau P_tau
            // 2^(55 - 8 tau), tau = 2..8 (levels 2..6 exact integers, 7 and 8
            // folded in FP32), in registers. Each level is released as soon as
            // it is read, so the next tile's MMAs into it (issued level by
            // level in the same order) start while the rest drains: levels 7
            // and 8 first (folded together), then 2..6. The products and row
            // sums below then run alongside the next tile's MMAs.
            int64_t wfix[kGroupLookups];
#pragma unroll
            for (int c0 = 0; c0 < kGroupLookups; c0 += kRedChunk) {
                const int l0 = group * kGroupLookups + c0;
                uint32_t p7[8], p8[8];
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                             : "=r"(p7[0]), "=r"(p7[1]), "=r"(p7[2]), "=r"(p7[3]), "=r"(p7[4]), "=r"(p7[5]),
                               "=r"(p7[6]), "=r"(p7[7])
                             : "r"(lane_base + 5 * kTileN + l0));
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                             : "=r"(p8[0]), "=r"(p8[1]), "=r"(p8[2]), "=r"(p8[3]), "=r"(p8[4]), "=r"(p8[5]),
                               "=r"(p8[6]), "=r"(p8[7])
                             : "r"(lane_base + 6 * kTileN + l0));
                asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
                for (int j = 0; j < kRedChunk; ++j)
                    wfix[c0 + j] = __float2int_rn(
                        fmaf(__uint_as_float(p8[j]), 0.001953125f, __uint_as_float(p7[j]) * 0.5f));
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            mbar_arrive(&sh.acc_empty[5]);
            mbar_arrive(&sh.acc_empty[6]);
#pragma unroll
            for (int lev = 0; lev < 5; ++lev) {
                uint32_t v[kGroupLookups / kRedChunk][8];
#pragma unroll
                for (int q = 0; q < kGroupLookups / kRedChunk; ++q) {
                    const uint32_t addr = lane_base + lev * kTileN + group * kGroupLookups + q * kRedChunk;
                    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                                 : "=r"(v[q][0]), "=r"(v[q][1]), "=r"(v[q][2]), "=r"(v[q][3]), "=r"(v[q][4]),
                                   "=r"(v[q][5]), "=r"(v[q][6]), "=r"(v[q][7])
                                 : "r"(addr));
                }
                asm volatile("tcgen05.wait::ld.sync.aligned;");
                const int shift = 39 - 8 * lev;  // 2^(55 - 8 tau), tau = lev + 2
#pragma unroll
                for (int q = 0; q < kGroupLookups / kRedChunk; ++q)
#pragma unroll
                    for (int j = 0; j < kRedChunk; ++j)
                        wfix[q * kRedChunk + j] +=
                            static_cast<int64_t>(__float2int_rn(__uint_as_float(v[q][j]))) * (int64_t{1} << shift);
                asm volatile("tcgen05.fence::before_thread_sync;");
                mbar_arrive(&sh.acc_empty[lev]);  // this level may take the next tile's MMAs
            }
#pragma unroll
            for (int c0 = 0; c0 < kGroupLookups; c0 += kRedChunk) {
                const int l0 = group * kGroupLookups + c0;
#pragma unroll
                for (int j = 0; j < kRedChunk; ++j) {
                    const int l = l0 + j;
                    const int64_t tf = sh.ubasis[l * kRows + (row ^ (l & 31))];
                    const uint64_t lo = static_cast<uint64_t>(wfix[c0 + j]) * static_cast<uint64_t>(tf);
                    int64_t hi = __mul64hi(wfix[c0 + j], tf);
                    const uint64_t lo2 = lo + (uint64_t{1} << 61);
                    hi += lo2 < lo ? 1 : 0;
                    red[j * kRows + row] = static_cast<int64_t>((static_cast<uint64_t>(hi) << 2) | (lo2 >> 62));
                }
                group_sync(group);
                // 16 threads per lookup sum 8 rows each (rows part + 16 i), then 4 shuffle levels
                {
                    const int j = row >> 4, part = row & 15;
                    uint64_t slo = 0;
                    int64_t shi = 0;
#pragma unroll
                    for (int i = 0; i < kRows / 16; ++i) {
                        const int64_t t = red[j * kRows + part + 16 * i];
                        const uint64_t nlo = slo + static_cast<uint64_t>(t);
                        shi += (t < 0 ? -1 : 0) + (nlo < slo ? 1 : 0);
                        slo = nlo;
                    }
#pragma unroll
                    for (int off = 8; off > 0; off >>= 1) {
                        const uint64_t olo = __shfl_xor_sync(0xffffffffu, slo, off);
                        const int64_t ohi = __shfl_xor_sync(0xffffffffu, shi, off);
                        const uint64_t nlo = slo + olo;
                        shi += ohi + (nlo < slo ? 1 : 0);
                        slo = nlo;
                    }
                    if (part == 0) {
                        sh.sums[l0 + j][0] = static_cast<int64_t>(slo);
                        sh.sums[l0 + j][1] = shi;
                    }
                }
                group_sync(group);
            }
            // finalisation: the group's first warp, one lookup per lane, so
            // that the few FP64 operations are issued once per 32 lookups. A
            // block of several sub-blocks leaves its exact 128-bit part for
            // the combine kernel instead.
            const int l = group * kGroupLookups + row;
            if (row < kGroupLookups && static_cast<uint32_t>(l) < count) {
                const uint64_t info = meta.info[l];
                if constexpr (!Chunked) {
                    store_green(p, w, info,
                                int128_to_double(sh.sums[l][1], static_cast<uint64_t>(sh.sums[l][0]), exponent - 55));
                } else {
                    const int64_t slot = part_slot(info, plan, nmax, meta.sub);
                    parts[2 * slot] = sh.sums[l][0];
                    parts[2 * slot + 1] = sh.sums[l][1];
                }
            }
            group_sync(group);  // sums are reused by the next tile
            mbar_arrive(&sh.meta_empty[mb]);
        }
    } else if (warp == kWarpCopy) {
        // ----------------------------------------- coefficient streaming --
        if (lane == 0) {
            uint32_t a_cnt = 0;
            unsigned long long streamed = 0;
            for (uint32_t tile = tile_begin; tile < tile_end && !failed(sh); ++tile) {
                const TileSource src = tile_source<Chunked>(plan, tiles[tile].block);
                for (int ks = 0; ks < src.ksteps; ++ks, ++a_cnt) {
                    const int st = static_cast<int>(a_cnt % kAStages);
                    if (a_cnt >= kAStages && !mbar_wait(&sh.a_empty[st], ((a_cnt / kAStages) - 1) & 1)) {
                        sh.error = 1;
                        break;
                    }
                    mbar_expect_tx(&sh.a_full[st], kAStageBytes);
                    bulk_copy_g2s(sh.a_ring[st], src.a + static_cast<int64_t>(ks) * (kAStageBytes / 2),
                                  kAStageBytes, &sh.a_full[st]);
                    streamed += kAStageBytes;
                }
            }
            if (counters) atomicAdd(counters + 1, streamed);
            // copies still in flight (only after an error) land before the CTA exits
            for (uint32_t st = 0; st < static_cast<uint32_t>(kAStages); ++st) {
                if (a_cnt <= st) continue;
                const uint32_t last = a_cnt - 1 - (a_cnt - 1 - st) % kAStages;
                if (!mbar_wait(&sh.a_full[st], (last / kAStages) & 1)) sh.error = 1;
            }
        }
    } else if (warp == kWarpMma) {
        // ---------------------------------------------------- MMA issue --
        if (lane == 0) {
            const uint32_t idesc = mma_idesc(kRows, kTileN);
            uint32_t a_cnt = 0, b_cnt = 0, tile_cnt = 0;
            unsigned long long mmas = 0;
            bool ok = true, issued = false;
            // with several column chunks the K steps vary by tile: the next
            // tile's key is loaded while this one's MMAs are issued
            const bool chunked = Chunked && plan.nkc > 1;
            uint32_t next_key = chunked && tile_begin < tile_end ? tiles[tile_begin].block : 0;
            for (uint32_t tile = tile_begin; ok && tile < tile_end && !failed(sh); ++tile, ++tile_cnt) {
                const uint32_t key = next_key;
                if (chunked && tile + 1 < tile_end) next_key = tiles[tile + 1].block;
                const int ksteps = chunked ? chunk_ksteps(plan, tile_kc(plan, key)) : plan.ksteps_last;
                for (int ks = 0; ok && ks < ksteps; ++ks, ++a_cnt, ++b_cnt) {
                    const int sa = static_cast<int>(a_cnt % kAStages);
                    const int sb = static_cast<int>(b_cnt % kBStages);
                    if (!mbar_wait(&sh.a_full[sa], (a_cnt / kAStages) & 1) ||
                        !mbar_wait(&sh.b_full[sb], (b_cnt / kBStages) & 1)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    // descriptors of the stage's first slices; a slice further
                    // on is the same descriptor plus its byte offset / 16 (the
                    // 14-bit address field cannot carry: shared memory < 256 KiB)
                    const uint64_t a_desc = smem_desc(smem_addr(sh.a_ring[sa]), 128, 256);
                    const uint64_t b_desc = smem_desc(smem_addr(sh.b_ring[sb]), 128, 256);
                    const uint32_t first = ks > 0 ? 1u : 0u;
                    // Issue order: the 29 MMAs of a K step interleaved so that two
                    // MMAs into the same accumulator are at least 3 apart, also
                    // across consecutive K steps (an MMA waits for the previous
                    // one into its accumulator). In a tile's first K step the
                    // accumulators are taken as the epilogue releases them:
                    // levels 7 and 8 (in the same interleaved order), then 2..6
                    // one level at a time. Within a level the pairs are always in
                    // increasing t (t = 8: the eighth digit, last), so each
                    // accumulator sums its products in the same order.
                    constexpr int kIssue = 29;
                    constexpr int8_t kIssueT[kIssue] = {1, 1, 1, 1, 1, 2, 2, 1, 2, 3, 2, 2, 3, 4, 3,
                                                        1, 5, 4, 3, 4, 3, 6, 2, 5, 7, 5, 4, 6, 8};
                    constexpr int8_t kIssueTp[kIssue] = {3, 5, 7, 6, 4, 6, 4, 2, 5, 5, 2, 3, 4, 4, 3,
                                                         1, 3, 3, 2, 2, 1, 2, 1, 2, 1, 1, 1, 1, 1};
                    auto mma_pair = [&](int t, int tp) {
                        const int level = t + tp - 2;
                        mma_f16(tmem + level * kTileN, a_desc + (t - 1) * (kRows * kKStep * 2 / 16),
                                b_desc + (tp - 1) * (kTileN * kKStep * 2 / 16), idesc, t > 1 ? 1u : first);
                    };
                    auto mma_eighth = [&]() {
                        mma_f16(tmem + (kLevels - 1) * kTileN, a_desc + kSlices * (kRows * kKStep * 2 / 16), b_desc,
                                idesc, 1u);
                    };
                    if (ks == 0 && tile_cnt > 0) {
                        ok = mbar_wait(&sh.acc_empty[kLevels - 2], (tile_cnt - 1) & 1) &&
                             mbar_wait(&sh.acc_empty[kLevels - 1], (tile_cnt - 1) & 1);
                        if (!ok) break;
                        asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
                        for (int i = 0; i < kIssue; ++i) {
                            if (kIssueT[i] == 8) mma_eighth();
                            else if (kIssueT[i] + kIssueTp[i] - 2 >= kLevels - 2) mma_pair(kIssueT[i], kIssueTp[i]);
                        }
                        issued = true;
#pragma unroll
                        for (int level = 0; level < kLevels - 2 && ok; ++level) {
                            ok = mbar_wait(&sh.acc_empty[level], (tile_cnt - 1) & 1);
                            if (!ok) break;
                            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
                            for (int t = 1; t <= level + 1; ++t) mma_pair(t, level + 2 - t);
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < kIssue; ++i) {
                            if (kIssueT[i] == 8) mma_eighth();
                            else mma_pair(kIssueT[i], kIssueTp[i]);
                        }
                    }
                    issued = true;
                    if (!ok) break;
                    mmas += kIssue;
                    mma_commit(&sh.a_empty[sa]);
                    mma_commit(&sh.b_empty[sb]);
                }
                if (!ok) break;
                mma_commit(&sh.acc_full);
            }
            if (!ok) sh.error = 1;
            if (counters) atomicAdd(counters, mmas);
            // every MMA issued has completed before the columns are freed
            if (issued) {
                mma_commit(&sh.drain);
                if (!mbar_wait(&sh.drain, 0)) sh.error = 1;
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (tid == 0 && sh.error) atomicExch(error_flag, 1);
    if (warp == kWarpMma) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
    }
}

// One thread per (configuration, i, j) of a table with several sub-blocks per
// coefficient block: each lookup's parts, exact 128-bit integers on the
// block's common scale, are summed (exactly, so the order does not matter)
// and rounded once, then stored as the single-sub-block finalisation does.
__global__ void __launch_bounds__(128) split_combine(const __grid_constant__ Problem p,
                                                     const __grid_constant__ Scratch w,
                                                     const __grid_constant__ SplitPlan plan,
                                                     const SplitRecordArrays rec,
                                                     const int64_t* __restrict__ parts) {
    const int64_t per_c = static_cast<int64_t>(p.max_order) * p.max_order;
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= p.batch * per_c) return;
    const int nsub = plan.nrb * plan.nkc;
    const int rpp = records_per_pair(plan);
    for (int k = 0; k < rpp; ++k) {
        const int64_t base = (idx * rpp + k) * nsub;
        const uint32_t key = rec.key[base];
        if (key == kNoKey) continue;
        uint64_t lo = 0;
        int64_t hi = 0;
        for (int sub = 0; sub < nsub; ++sub) {
            const uint64_t plo = static_cast<uint64_t>(parts[2 * (base + sub)]);
            const uint64_t nlo = lo + plo;
            hi += parts[2 * (base + sub) + 1] + (nlo < lo ? 1 : 0);
            lo = nlo;
        }
        store_green(p, w, rec.info[base], int128_to_double(hi, lo, tile_source<true>(plan, key).exponent - 55));
    }
}

}  // namespace

void split_geometry(int nu, int nv, int* nrb, int* nkc, int* ksteps_last) {
    *nrb = (nu + kRows - 1) / kRows;
    *nkc = (nv + kSubK - 1) / kSubK;
    *ksteps_last = (nv - (*nkc - 1) * kSubK + kKStep - 1) / kKStep;
}

size_t split_slices_bytes(int nu, int nv, size_t blocks) {
    int nrb, nkc, ksteps_last;
    split_geometry(nu, nv, &nrb, &nkc, &ksteps_last);
    return blocks * nrb * static_cast<size_t>(row_ksteps(nkc, ksteps_last)) * kAStageBytes;
}

cudaError_t launch_slice_table(const double* coeffs, int nu, int nv, size_t blocks, uint16_t* slices,
                               int32_t* exponents, cudaStream_t stream) {
    if (blocks == 0) return cudaSuccess;
    int nrb, nkc, ksteps_last;
    split_geometry(nu, nv, &nrb, &nkc, &ksteps_last);
    const size_t grid = blocks * nrb * nkc;
    if (grid > 0x7FFFFFFFu) return cudaErrorInvalidValue;
    slice_blocks<<<static_cast<unsigned>(grid), 256, 0, stream>>>(coeffs, nu, nv, nrb, nkc, ksteps_last, slices,
                                                                  exponents);
    return cudaGetLastError();
}

size_t split_scratch_bytes(int64_t batch, int max_order, const SplitPlan& plan) {
    const size_t nsub = static_cast<size_t>(plan.nrb) * plan.nkc;
    const size_t nrec = static_cast<size_t>(batch) * max_order * max_order * records_per_pair(plan) * nsub;
    size_t total = 0;
    total += nrec * (4 + 8 + 8 + 8);          // unsorted records
    total += nrec * (8 + 8 + 8);              // sorted records
    total += static_cast<size_t>(plan.nblocks) * 4 * 4;  // counts, offsets, tile offsets, cursors
    total += (nrec / kTileN + plan.nblocks + 1) * sizeof(SplitTile);  // tiles
    if (nsub > 1) total += nrec * 16;         // 128-bit sub-block parts
    total += 16 + kSplitStatusBytes;          // totals, error flag and counters
    return total + 16 * 256;
}

cudaError_t launch_split_assembly(const Problem& p, const Scratch& w, const SplitPlan& plan, void* scratch,
                                  size_t scratch_bytes, int sm_count, int32_t** error_flag_out,
                                  cudaStream_t stream, const KernelEvents* events) {
    const int64_t pairs = p.batch * static_cast<int64_t>(p.max_order) * p.max_order;
    const int nsub = plan.nrb * plan.nkc;
    const int64_t nrec = pairs * records_per_pair(plan) * nsub;
    char* cursor = static_cast<char*>(scratch);
    auto take = [&](size_t bytes) {
        void* ptr = cursor;
        cursor += (bytes + 255) & ~static_cast<size_t>(255);
        return ptr;
    };
    SplitRecordArrays rec{static_cast<uint32_t*>(take(nrec * 4)), static_cast<double*>(take(nrec * 8)),
                          static_cast<double*>(take(nrec * 8)), static_cast<uint64_t*>(take(nrec * 8))};
    SplitRecordArrays sorted{nullptr, static_cast<double*>(take(nrec * 8)), static_cast<double*>(take(nrec * 8)),
                             static_cast<uint64_t*>(take(nrec * 8))};
    uint32_t* counts = static_cast<uint32_t*>(take(plan.nblocks * 4u));
    uint32_t* offsets = static_cast<uint32_t*>(take(plan.nblocks * 4u));
    uint32_t* tile_offsets = static_cast<uint32_t*>(take(plan.nblocks * 4u));
    uint32_t* cursors = static_cast<uint32_t*>(take(plan.nblocks * 4u));
    SplitTile* tiles = static_cast<SplitTile*>(take((nrec / kTileN + plan.nblocks + 1) * sizeof(SplitTile)));
    int64_t* parts = nsub > 1 ? static_cast<int64_t*>(take(nrec * 16)) : nullptr;
    uint32_t* totals = static_cast<uint32_t*>(take(16));
    // the error flag (int32 at byte 0) and the assembly's counters (uint64 at
    // bytes 8 and 16: MMAs issued, coefficient-slice bytes streamed)
    int32_t* error_flag = static_cast<int32_t*>(take(kSplitStatusBytes));
    unsigned long long* counters = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(error_flag) + 8);
    if (static_cast<size_t>(cursor - static_cast<char*>(scratch)) > scratch_bytes) return cudaErrorInvalidValue;
    if (error_flag_out) *error_flag_out = error_flag;

    cudaError_t err = cudaMemsetAsync(counts, 0, plan.nblocks * 4u, stream);
    if (err != cudaSuccess) return err;
    err = cudaMemsetAsync(error_flag, 0, kSplitStatusBytes, stream);
    if (err != cudaSuccess) return err;
    split_descriptors<<<static_cast<unsigned>((pairs + 127) / 128), 128, 0, stream>>>(p, w, plan, rec, counts);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    split_scan<<<1, 1024, 0, stream>>>(counts, plan.nblocks, offsets, tile_offsets, cursors, totals);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    split_scatter<<<static_cast<unsigned>((nrec + 255) / 256), 256, 0, stream>>>(rec, nrec, offsets, cursors,
                                                                                 sorted);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    split_tiles<<<(plan.nblocks + 255) / 256, 256, 0, stream>>>(counts, plan.nblocks, offsets, tile_offsets,
                                                                tiles);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    if (events && events->marks[1]) cudaEventRecord(events->marks[1], stream);
    const size_t smem = sizeof(SplitShared);
    auto kernel = nsub > 1 ? split_assembly<true> : split_assembly<false>;
    err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (err != cudaSuccess) return err;
    kernel<<<sm_count, kAssemblyThreads, smem, stream>>>(p, w, plan, sorted, tiles, totals, parts, error_flag,
                                                         counters);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    if (nsub > 1) {
        split_combine<<<static_cast<unsigned>((pairs + 127) / 128), 128, 0, stream>>>(p, w, plan, rec, parts);
        err = cudaGetLastError();
    }
    return err;
}

}  // namespace cdet
