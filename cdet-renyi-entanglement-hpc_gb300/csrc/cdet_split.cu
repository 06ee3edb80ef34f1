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
constexpr int kTileN = 128;         // lookups per tile (MMA M: TMEM lanes)
constexpr int kRows = 128;          // coefficient rows a of a sub-block (MMA N at most, zero padded)
constexpr int kKStep = 16;          // MMA K (bf16)
constexpr int kSubKSteps = kSubK / kKStep;  // K steps of a full column chunk
constexpr long long kWaitCycles = 2000000000LL;  // ~1 s at 2 GHz: bound of every mbarrier wait

// bytes of one slice of either operand: 128 rows x 16 k x fp16
constexpr uint32_t kSliceBytes = kRows * kKStep * 2;                  // 4 KiB
// bytes of the coefficient operand of one K step: 8 slices x 128 rows x 16 k x fp16
constexpr uint32_t kAStageBytes = kSlicesA * kSliceBytes;             // 32 KiB
// bytes of the basis operand of one K step: 7 slices x 128 lookups x 16 k x fp16
constexpr uint32_t kBStepBytes = kSlices * kTileN * kKStep * 2;       // 28 KiB
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

// Each K step also records its lead: the first slice t (1..8) holding a
// nonzero digit in any of its 128 rows x 16 columns, 9 when all are zero.
// Chebyshev coefficients decay with the degree, so the high K steps of a
// block hold only low-weight digits: a product with a slice before the lead
// is exactly zero and the assembly neither streams nor multiplies it.
// leads[(block * nrb + rb) * row_ksteps + ks], one byte per K step.
// Each sub-block also records its level rows: for each accumulator level
// tau = 2..8, the number of leading rows that have a digit able to reach it
// (rows with a nonzero digit t <= tau - 1; for tau = 8 also the eighth
// digit), byte tau - 2 of level_rows[block * nrb * nkc + sub]. Rows below
// that count contribute exactly zero to the level.
__global__ void __launch_bounds__(256) slice_blocks(const double* __restrict__ coeffs, int nu, int nv,
                                                    int nrb, int nkc, int ksteps_last,
                                                    uint16_t* __restrict__ out, int32_t* __restrict__ exponents,
                                                    uint8_t* __restrict__ leads, uint64_t* __restrict__ level_rows) {
    const int nsub = nrb * nkc;
    const int64_t block = blockIdx.x / nsub;
    const int sub = static_cast<int>(blockIdx.x - block * nsub);
    const int rb = sub / nkc, kc = sub - (sub / nkc) * nkc;
    const int row0 = rb * kRows, col0 = kc * kSubK;
    const int ksteps = kc == nkc - 1 ? ksteps_last : kSubKSteps;
    const int rk = row_ksteps(nkc, ksteps_last);
    const double* c = coeffs + block * static_cast<int64_t>(nu) * nv;
    __shared__ double red[256];
    __shared__ int s_lead[kSubKSteps];
    __shared__ int s_row_lead[kRows];
    __shared__ int s_level_rows[kLevels];
    if (threadIdx.x < kSubKSteps) s_lead[threadIdx.x] = kSlicesA + 1;
    if (threadIdx.x < kRows) s_row_lead[threadIdx.x] = kSlicesA + 1;
    if (threadIdx.x < kLevels) s_level_rows[threadIdx.x] = 0;
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
    int lead[kSubKSteps];  // this thread's first nonzero slice per K step
#pragma unroll
    for (int ks = 0; ks < kSubKSteps; ++ks) lead[ks] = kSlicesA + 1;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
        const int a = i / (ksteps * kKStep);
        const int b = i - a * (ksteps * kKStep);
        const int ag = row0 + a, bg = col0 + b;
        double r = (ag < nu && bg < nv) ? ldexp(c[ag * nv + bg], -e) : 0.0;  // |r| < 1
        const int ks = b / kKStep, bb = b - ks * kKStep;
        const int k = (bb & 1) * 8 + (bb >> 1);
        uint16_t* base = dst + static_cast<int64_t>(ks) * kSlicesA * kRows * kKStep + core_offset(a, k);
        int first = kSlicesA + 1;
        for (int t = 0; t < kSlicesA; ++t) {
            // exact: r * 256 has the same significand, and subtracting the
            // nearest integer leaves the (representable) remainder
            const double scaled = r * 256.0;
            const double q = rint(scaled);
            r = scaled - q;
            if (q != 0.0 && first > kSlicesA) first = t + 1;
            const float stored = t < kSlicesA - 1 ? static_cast<float>(q) : static_cast<float>(q) * 0.00390625f;
            base[t * kRows * kKStep] = __half_as_ushort(__float2half_rn(stored));
        }
#pragma unroll
        for (int q = 0; q < kSubKSteps; ++q)
            if (q == ks) lead[q] = min(lead[q], first);
        if (first <= kSlicesA) atomicMin(&s_row_lead[a], first);
    }
#pragma unroll
    for (int q = 0; q < kSubKSteps; ++q) {
        int v = lead[q];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, off));
        if ((threadIdx.x & 31) == 0 && v <= kSlicesA) atomicMin(&s_lead[q], v);
    }
    __syncthreads();
    if (threadIdx.x < static_cast<unsigned>(ksteps))
        leads[(block * nrb + rb) * rk + static_cast<int64_t>(kc) * kSubKSteps + threadIdx.x] =
            static_cast<uint8_t>(s_lead[threadIdx.x]);
    if (threadIdx.x < kRows) {
        const int rl = s_row_lead[threadIdx.x];
#pragma unroll
        for (int lv = 0; lv < kLevels; ++lv) {
            // level tau = lv + 2 takes digits t <= tau - 1 (and, at tau = 8, the eighth)
            const int reach = lv == kLevels - 1 ? kSlicesA : lv + 1;
            if (rl <= reach) atomicMax(&s_level_rows[lv], static_cast<int>(threadIdx.x) + 1);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t packed = 0;
        for (int lv = 0; lv < kLevels; ++lv) packed |= static_cast<uint64_t>(s_level_rows[lv]) << (8 * lv);
        level_rows[block * nsub + sub] = packed;
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

// A lookup after the sort by sub-block: one 32-byte record, so that the
// scatter writes one sector per lookup (its positions are scattered).
struct __align__(32) SortedLookup {
    double u, v;
    uint64_t info, pad;
};

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

// Configurations per warp of split_descriptors: as many whole
// configurations' vertices as 32 lanes hold (max_order <= 24).
__host__ __device__ inline int descriptor_configs_per_warp(int nmax) { return nmax >= 1 && nmax <= 32 ? 32 / nmax : 1; }

// One warp per K = 32 / max_order configurations (at least one): each
// vertex is decoded once, on its lane (tau = beta u_tau, the site and
// replica indices, and u = 2 tau / beta - 1, the vertex's value when it is
// the outer one of a pair), then the warp takes the vertex pairs 32 at a time,
// the two vertices' values by shuffles, and computes per pair only v = 2
// tau_inner / tau_outer - 1 (the same operations as per-pair decoding, so the
// same values). Branch and (u, v) are shared by both table sets; the corner
// path is evaluated here, every other lookup becomes one record per sub-block
// of its coefficient block, keyed by the sub-block. Record slots are fixed:
// ((c * nmax^2 + pair) * records_per_pair + record) * nsub + sub, the set's
// records after those of the sets before it.
__global__ void __launch_bounds__(128) split_descriptors(const __grid_constant__ Problem p,
                                                         const __grid_constant__ Scratch w,
                                                         const __grid_constant__ SplitPlan plan,
                                                         SplitRecordArrays rec, uint32_t* counts) {
    const int nmax = p.max_order;
    const int per_c = nmax * nmax;
    const int K = descriptor_configs_per_warp(nmax);
    const int lane = threadIdx.x & 31;
    const int64_t c0 = ((static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5) * K;
    if (c0 >= p.batch) return;  // the whole warp
    const Scalars& s = p.s;
    const int nsub = plan.nrb * plan.nkc;
    const int rpp = records_per_pair(plan);
    // this lane's vertex: vertex vv of configuration c0 + vc
    const int vc = lane / nmax, vv = lane - (lane / nmax) * nmax;
    const int64_t cv = c0 + vc;
    int nv = 0, xv = 0, yv = 0, rv = 0;
    bool vbad = false;
    double tuv = 0.0, tauv = 0.0, uv = 0.0;
    if (vc < K && cv < p.batch) {
        nv = p.all_subsets ? nmax : __ldg(p.orders + cv);
        if (nv >= 1 && nv <= nmax && vv < nv) {
            const double* vb = p.vertices + (cv * nmax + vv) * 4;
            tuv = __ldg(vb);
            if (!isfinite(tuv)) vbad = true;
            tauv = dmul(s.beta, tuv);
            xv = coordinate_index_s(dmul(static_cast<double>(s.n1), __ldg(vb + 1)), s.n1, vbad);
            yv = coordinate_index_s(dmul(static_cast<double>(s.n2), __ldg(vb + 2)), s.n2, vbad);
            rv = coordinate_index_s(dmul(2.0, __ldg(vb + 3)), 2, vbad);
            uv = clamp_unit_s(dsub(ddiv(dmul(2.0, tauv), s.beta), 1.0));
        }
    }
    const int total = K * per_c;
    for (int q0 = 0; q0 < total; q0 += 32) {
        const int q = q0 + lane;
        const bool valid = q < total;
        const int cq = valid ? q / per_c : 0;
        const int pair = valid ? q - cq * per_c : 0;
        const int i = pair / nmax, j = pair - (pair / nmax) * nmax;
        const int li = cq * nmax + i, lj = cq * nmax + j;  // the two vertices' lanes (< K nmax <= 32)
        const int n = __shfl_sync(0xffffffffu, nv, li);
        const double tui = __shfl_sync(0xffffffffu, tuv, li), tuj = __shfl_sync(0xffffffffu, tuv, lj);
        const double taui = __shfl_sync(0xffffffffu, tauv, li), tauj = __shfl_sync(0xffffffffu, tauv, lj);
        const double ui = __shfl_sync(0xffffffffu, uv, li), uj = __shfl_sync(0xffffffffu, uv, lj);
        const int xi = __shfl_sync(0xffffffffu, xv, li), xj = __shfl_sync(0xffffffffu, xv, lj);
        const int yi = __shfl_sync(0xffffffffu, yv, li), yj = __shfl_sync(0xffffffffu, yv, lj);
        const int ri = __shfl_sync(0xffffffffu, rv, li), rj = __shfl_sync(0xffffffffu, rv, lj);
        const bool bad = __shfl_sync(0xffffffffu, static_cast<int>(vbad), li) != 0 ||
                         __shfl_sync(0xffffffffu, static_cast<int>(vbad), lj) != 0;
        const int64_t c = c0 + cq;
        if (!valid || c >= p.batch) continue;
        const int64_t slot0 = (c * per_c + pair) * rpp * nsub;
        for (int k = 0; k < rpp * nsub; ++k) rec.key[slot0 + k] = kNoKey;
        if (n < 1 || n > nmax) {
            if (pair == 0) atomicOr(p.status + c, kStatusBadInput);
            continue;
        }
        if (i >= n || j >= n) continue;
        if (bad) {
            atomicOr(p.status + c, kStatusBadInput);
            continue;
        }
        if (copy_reused_pair(p, w.green, w.diag, c, 0, i, j, n)) {  // both vertices retained: no records
            copy_reused_pair(p, w.green, w.diag, c, 1, i, j, n);
            continue;
        }
        const bool upper = (i != j) && (tui > tuj);
        const double t_outer = upper ? taui : tauj;
        const double t_inner = upper ? tauj : taui;
        const bool corner = t_outer < s.branch_eps;
        double u = 0.0, v = 0.0;
        if (!corner) {
            u = upper ? ui : uj;  // clamp(2 t_outer / beta - 1), decoded with the outer vertex
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
                    const double up_raw = up, down_raw = down;
                    up = dadd(up, s.diag_up_shift);
                    down = dadd(down, s.diag_down_shift);
                    w.diag[mslot * nmax + i] = p.raw_diag ? up_raw : up;
                    w.diag[(mslot + 1) * nmax + i] = p.raw_diag ? down_raw : down;
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
}

// Exclusive scan of block counts (offsets) and of their 128-lookup tile counts
// (tile offsets); one CTA of 1024 threads. totals[0] = lookups, totals[1] = tiles.
// The estimated time of one tile of sub-block `key` (its branch's key_costs).
__device__ __forceinline__ uint32_t key_cost(const SplitPlan& plan, uint32_t key) {
    int seg = 0;
    while (seg + 1 < plan.segments && key >= plan.segment_base[seg + 1]) ++seg;
    return __ldg(plan.key_costs[seg] + (key - plan.segment_base[seg]));
}

// Exclusive scans over the keys of their lookup counts (offsets), tile counts
// (tile_offsets) and estimated tile time (cost_prefix: tiles x key cost);
// totals[0] = lookups, totals[1] = tiles, totals[2..3] = the time as uint64.
// One block of 32 warps, each a contiguous chunk of the keys read 32 at a
// time (coalesced), a warp scan by shuffles carrying the running sums.
struct KeySums {
    uint32_t lookups, tiles;
    unsigned long long cost;
};

__device__ __forceinline__ KeySums key_sums(const SplitPlan& plan, const uint32_t* counts, uint32_t b, uint32_t end) {
    KeySums k{0, 0, 0};
    if (b < end) {
        k.lookups = counts[b];
        k.tiles = (k.lookups + kTileN - 1) / kTileN;
        if (k.tiles) k.cost = static_cast<unsigned long long>(k.tiles) * key_cost(plan, b);
    }
    return k;
}

__global__ void __launch_bounds__(1024) split_scan(const SplitPlan plan, const uint32_t* __restrict__ counts,
                                                   uint32_t* __restrict__ offsets,
                                                   uint32_t* __restrict__ tile_offsets,
                                                   uint32_t* __restrict__ cursors,
                                                   unsigned long long* __restrict__ cost_prefix,
                                                   uint32_t* __restrict__ totals) {
    __shared__ KeySums s_warp[32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nblocks = plan.nblocks;
    const uint32_t chunk = ((nblocks + 32 * 32 - 1) / (32 * 32)) * 32;  // keys per warp, a multiple of 32
    const uint32_t begin = min(nblocks, warp * chunk), end = min(nblocks, begin + chunk);
    // pass 1: the warp's sums
    KeySums mine{0, 0, 0};
    for (uint32_t b = begin + lane; b < end; b += 32) {
        const KeySums k = key_sums(plan, counts, b, end);
        mine.lookups += k.lookups;
        mine.tiles += k.tiles;
        mine.cost += k.cost;
    }
    for (int off = 16; off > 0; off >>= 1) {
        mine.lookups += __shfl_xor_sync(0xffffffffu, mine.lookups, off);
        mine.tiles += __shfl_xor_sync(0xffffffffu, mine.tiles, off);
        mine.cost += __shfl_xor_sync(0xffffffffu, mine.cost, off);
    }
    if (lane == 0) s_warp[warp] = mine;
    __syncthreads();
    KeySums run{0, 0, 0};
    for (int w = 0; w < warp; ++w) {
        run.lookups += s_warp[w].lookups;
        run.tiles += s_warp[w].tiles;
        run.cost += s_warp[w].cost;
    }
    if (threadIdx.x == 0) {
        KeySums all{0, 0, 0};
        for (int w = 0; w < 32; ++w) {
            all.lookups += s_warp[w].lookups;
            all.tiles += s_warp[w].tiles;
            all.cost += s_warp[w].cost;
        }
        totals[0] = all.lookups;
        totals[1] = all.tiles;
        *reinterpret_cast<unsigned long long*>(totals + 2) = all.cost;
    }
    // pass 2: the exclusive prefixes, 32 keys a round
    KeySums next = key_sums(plan, counts, begin + lane, end);
    for (uint32_t b0 = begin; b0 < end; b0 += 32) {
        const KeySums k = next;
        next = key_sums(plan, counts, b0 + 32 + lane, end);  // the next round's keys, in flight meanwhile
        KeySums incl = k;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t a = __shfl_up_sync(0xffffffffu, incl.lookups, off);
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl.tiles, off);
            const unsigned long long c = __shfl_up_sync(0xffffffffu, incl.cost, off);
            if (lane >= off) {
                incl.lookups += a;
                incl.tiles += t;
                incl.cost += c;
            }
        }
        const uint32_t b = b0 + lane;
        if (b < end) {
            offsets[b] = run.lookups + incl.lookups - k.lookups;
            tile_offsets[b] = run.tiles + incl.tiles - k.tiles;
            cost_prefix[b] = run.cost + incl.cost - k.cost;
            cursors[b] = 0;
        }
        run.lookups += __shfl_sync(0xffffffffu, incl.lookups, 31);
        run.tiles += __shfl_sync(0xffffffffu, incl.tiles, 31);
        run.cost += __shfl_sync(0xffffffffu, incl.cost, 31);
    }
}

struct SplitTile {
    uint32_t block, start, count, pad;
};

// Scatter records into block order and emit the tile list.
__global__ void __launch_bounds__(256) split_scatter(const SplitRecordArrays rec, int64_t nrec,
                                                     const uint32_t* __restrict__ offsets,
                                                     uint32_t* __restrict__ cursors,
                                                     SortedLookup* __restrict__ sorted) {
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= nrec) return;
    const uint32_t key = rec.key[idx];
    if (key == kNoKey) return;
    const uint32_t pos = offsets[key] + atomicAdd(cursors + key, 1u);
    double2* out = reinterpret_cast<double2*>(sorted + pos);
    out[0] = make_double2(rec.u[idx], rec.v[idx]);
    reinterpret_cast<ulonglong2*>(out)[1] = make_ulonglong2(rec.info[idx], 0ull);
}


// ------------------------------------------------------------- assembly --
// Warp-specialised persistent kernel, one CTA of 14 warps per SM. A tile is
// up to 128 lookups of one sort key (one sub-block of one coefficient
// block). For every lookup l (a TMEM lane) and coefficient row a (a TMEM
// column) the MMAs accumulate, level by level, W[l][a] = sum_b T_b(v_l) C[a][b]:
//   warps 0-3   basis producers: thread l generates T_b(v_l) for the 16 b of
//               each K step (eight chains of stride 8) and writes the digit
//               slices the step's MMAs read into a three-stage ring (the
//               MMA's A operand: 128 lookups x 16 k per slice, whole 16-byte
//               core-matrix rows);
//   warps 4-11  epilogue, two groups of four warps: thread (group g, lane l)
//               owns lookup l and, of every 16 coefficient rows, the rows
//               4g..4g+3 and 8+4g..8+4g+3. It reads its rows' levels from
//               tensor memory, combines them in fixed point, multiplies by
//               T_a(u_l) from its own recurrences and sums over a in
//               registers; the two groups' sums are added at the tile's end;
//   warp 12     one thread streams the coefficient slices of every K step
//               (the MMA's B operand: the sub-block's rows x 16 k per slice)
//               into a three-stage ring with cp.async.bulk;
//   warp 13     one thread issues the MMAs (kind::f16, M = 128, K = 16) and
//               owns the 512 TMEM columns.
// Each level's accumulator spans only the rows whose coefficients have a
// digit that can reach that level (the sub-block's level rows, recorded at
// slicing): the high rows of a decaying Chebyshev block hold only
// low-weight digits, so the leading levels are narrow (MMA N = their rows).
// When the levels' columns exceed the 496 below the sink the tile runs as
// two passes, over rows 0..63 and 64..127. The accumulators are
// single-buffered: a pass's MMAs start when the epilogue has drained the
// previous pass.
//
// Where only the low-weight levels reach, 32-bit arithmetic suffices and the
// kernel uses it: a K step whose lead is 6 or more multiplies only basis
// digits 1 and 2, so from the first K step after which every lead is at
// least 6 the producers run their chains in Q30 (error ~2^-26 against the
// 2^-16 resolution those digits need); rows that no level below 7 reaches
// (|W| < 2^24 units of 2^-55) take their T_a(u) from Q30 chains, a 32 x 32
// product and a 64-bit sum.
constexpr int kCStages = 3;   // coefficient ring
constexpr int kBStages = 3;   // basis ring
constexpr int kMetaBufs = 2;
constexpr int kProducerWarps = 4;
constexpr int kEpilogueGroups = 2;
constexpr int kEpilogueWarps = 4 * kEpilogueGroups;
constexpr int kWarpCopy = kProducerWarps + kEpilogueWarps;
constexpr int kWarpMma = kWarpCopy + 1;
// 14 warps: each SM sub-partition (16K registers) holds four of them, which
// caps the kernel at 128 registers per thread
constexpr int kAssemblyThreads = (kWarpMma + 1) * 32;
constexpr int kTmemColumns = 512;
constexpr int kTmemSink = kTmemColumns - 16;  // 16 columns no level uses (the writes of empty levels)
constexpr uint32_t kEpiBarrier = 1;           // named barrier of all epilogue warps (votes)
constexpr int kTailLead = 6;                  // K steps from this lead on read basis digits 1 and 2 only
static_assert(kProducerWarps * 32 == kTileN, "one basis producer thread per lookup");


struct TileMeta {
    double u[kTileN];
    uint64_t info[kTileN];
    uint64_t rows;  // level rows of the tile's sub-block
    uint32_t count;
    int32_t exponent;
    int32_t sub;
    uint32_t pad;
};

struct SplitShared {
    alignas(1024) uint16_t coeff_ring[kCStages][kAStageBytes / 2];  // 3 x 32 KiB
    alignas(1024) uint16_t basis_ring[kBStages][kBStepBytes / 2];   // 3 x 28 KiB
    alignas(16) int64_t sums[kTileN][2];                             // second group's (lo, hi) per lookup
    TileMeta meta[kMetaBufs];
    uint32_t c_lead[kCStages];  // first coefficient slice streamed into each stage (written before its copy)
    uint64_t c_full[kCStages], c_empty[kCStages];
    uint64_t b_full[kBStages], b_empty[kBStages];
    uint64_t meta_full[kMetaBufs], meta_empty[kMetaBufs];
    uint64_t acc_full, acc_empty;
    uint64_t drain;  // last commit of the MMA thread, waited on before dealloc
    uint32_t tmem_base;
    uint32_t error;
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
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
// find their coefficient slices, K-step leads, level rows and block exponent,
// and the sub-block's place: sub = rb * nkc + kc covers rows 128 rb.. and
// columns 128 kc.. in `ksteps` K steps.
struct TileSource {
    const uint16_t* a;
    const uint8_t* leads;  // lead of each of the sub-block's K steps
    const uint64_t* rows;  // the sub-block's level rows
    const int32_t* exponent;
    int sub, rb, kc, ksteps;
};
template <bool Chunked>
__device__ __forceinline__ TileSource tile_source(const SplitPlan& plan, uint32_t key) {
    int seg = 0;
    while (seg + 1 < plan.segments && key >= plan.segment_base[seg + 1]) ++seg;
    const uint32_t local = key - plan.segment_base[seg];
    TileSource t;
    t.rows = plan.level_rows[seg] + local;
    if constexpr (!Chunked) {  // one sub-block per block
        t.sub = t.rb = t.kc = 0;
        t.ksteps = plan.ksteps_last;
        t.a = plan.slices[seg] + static_cast<int64_t>(local) * plan.ksteps_last * (kAStageBytes / 2);
        t.leads = plan.leads[seg] + static_cast<int64_t>(local) * plan.ksteps_last;
        t.exponent = plan.exponents[seg] + local;
        return t;
    }
    const uint32_t nsub = static_cast<uint32_t>(plan.nrb * plan.nkc);
    const uint32_t block = local / nsub;
    t.sub = static_cast<int>(local - block * nsub);
    t.rb = t.sub / plan.nkc;
    t.kc = t.sub - t.rb * plan.nkc;
    t.ksteps = t.kc == plan.nkc - 1 ? plan.ksteps_last : kSubKSteps;
    const int rk = row_ksteps(plan.nkc, plan.ksteps_last);
    const int64_t step0 = (static_cast<int64_t>(block) * plan.nrb + t.rb) * rk + static_cast<int64_t>(t.kc) * kSubKSteps;
    t.a = plan.slices[seg] + step0 * (kAStageBytes / 2);
    t.leads = plan.leads[seg] + step0;
    t.exponent = plan.exponents[seg] + block;
    return t;
}

// Lead of K step ks as the assembly uses it: a tile's first K step is always
// complete (its MMAs initialise every accumulator level), a K step with no
// nonzero digit still streams and multiplies the eighth slice.
__device__ __forceinline__ int step_lead(const uint8_t* leads, int ks) {
    return ks == 0 ? 1 : min(static_cast<int>(__ldg(leads + ks)), kSlicesA);
}

// The first K step from which every lead is kTailLead or more (ksteps when
// none): from there the basis digits 1 and 2 are all the MMAs read.
__device__ __forceinline__ int tail_kstep(const uint8_t* leads, int ksteps) {
    int first = ksteps;
    for (int ks = ksteps - 1; ks >= 1 && step_lead(leads, ks) >= kTailLead; --ks) first = ks;
    return first;
}

// Tensor-memory layout of one pass of a tile: level lv (tau = lv + 2) takes
// n[lv] columns (its rows from row0, rounded up to 16; 0 when no digit of
// the sub-block reaches it) from column col[lv]. A tile whose levels fit in
// the 496 columns below the sink is one pass over all rows; otherwise two
// passes over rows 0..63 and 64..127 (at most 7 x 64 = 448 columns each).
struct PassGeom {
    int npass, row0, cols;  // cols: the widest level's columns
    int n[kLevels], col[kLevels];
};
__device__ __forceinline__ PassGeom pass_geom(uint64_t packed, int pass) {
    PassGeom g;
    int rows[kLevels], total = 0;
#pragma unroll
    for (int lv = 0; lv < kLevels; ++lv) {
        rows[lv] = static_cast<int>((packed >> (8 * lv)) & 0xFFu);
        total += (rows[lv] + 15) & ~15;
    }
    g.npass = total <= kTmemSink ? 1 : 2;
    g.row0 = g.npass == 1 ? 0 : 64 * pass;
    const int span = g.npass == 1 ? kRows : 64;
    int c = 0;
    g.cols = 0;
#pragma unroll
    for (int lv = 0; lv < kLevels; ++lv) {
        const int r = min(max(rows[lv] - g.row0, 0), span);
        g.n[lv] = (r + 15) & ~15;
        g.col[lv] = c;
        c += g.n[lv];
        g.cols = max(g.cols, g.n[lv]);
    }
    return g;
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
            w.diag[(mslot + spin) * nmax + i] = p.raw_diag ? value : g;  // unshifted for the double-double order 1
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

// T_0 .. T_8 of x in Q62 fixed point by the stride-1 recurrence
// T_{k+1} = 2 x T_k - T_{k-1} (the start values of the chains below).
__device__ __forceinline__ void cheb_table8(int64_t xfix, int64_t (&t)[9]) {
    t[0] = int64_t{1} << 62;
    t[1] = xfix;
#pragma unroll
    for (int k = 1; k < 8; ++k) t[k + 1] = cheb_step_q62(xfix, t[k], t[k - 1]);
}

// Chains of stride 8: T_{m+8} = 2 T_8(x) T_m - T_{m-8}. A thread runs
// several 8-apart chains side by side, so their steps are independent
// instructions rather than one long dependent recurrence; each chain's
// rounding error grows like the square of its own step count. The Q62 form
// feeds the digits and the rows that need all 55 bits; the Q30 form (int32,
// 1 = 2^30) the ones that need about 25.
struct ChebChain {
    int64_t prev, cur;  // T_{m-8}, T_m in Q62
    __device__ __forceinline__ int64_t next(int64_t t8) {
        const int64_t t = cur;
        cur = cheb_step_q62(t8, cur, prev);
        prev = t;
        return t;
    }
};
__device__ __forceinline__ int32_t q62_to_q30(int64_t x) {
    return static_cast<int32_t>((x + (int64_t{1} << 31)) >> 32);
}
struct ChebChain30 {
    int32_t prev, cur;  // T_{m-8}, T_m in Q30
    __device__ __forceinline__ int32_t next(int32_t t8) {
        const int32_t t = cur;
        // round(2 T_8 T_m / 2^30) - T_{m-8}
        cur = static_cast<int32_t>((static_cast<int64_t>(t8) * cur + (int64_t{1} << 28)) >> 29) - prev;
        prev = t;
        return t;
    }
};

// Columns addr..addr + 3 and addr + 8..addr + 11 of this warp's 32 lanes
// from tensor memory (an epilogue thread's 8 columns of a 16-column chunk).
__device__ __forceinline__ void tmem_load_4x2(uint32_t addr, uint32_t (&v)[8]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%8];\n"
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%4,%5,%6,%7}, [%9];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
        : "r"(addr), "r"(addr + 8));
}

// The 29 digit-pair MMAs of a K step: coefficient slice t (8: the pre-scaled
// eighth digit) against basis slice t', interleaved so that two MMAs into
// the same accumulator are at least 3 apart; within a level the pairs are in
// increasing t (the eighth digit last), so each accumulator sums its
// products in the same order and its first MMA (t = 1, in a tile's first K
// step, which is always complete) initialises it.
constexpr int kIssue = 29;
__device__ constexpr int8_t kIssueT[kIssue] = {1, 1, 1, 1, 1, 2, 2, 1, 2, 3, 2, 2, 3, 4, 3,
                                               1, 5, 4, 3, 4, 3, 6, 2, 5, 7, 5, 4, 6, 8};
__device__ constexpr int8_t kIssueTp[kIssue] = {3, 5, 7, 6, 4, 6, 4, 2, 5, 5, 2, 3, 4, 4, 3,
                                                1, 3, 3, 2, 2, 1, 2, 1, 2, 1, 1, 1, 1, 1};

// One K step's MMAs with coefficient slices from Lead on, as straight-line
// code: every operand is in a register before the first MMA, so the single
// issuing thread puts them into the tensor pipe back to back (computing an
// operand or branching between two MMAs costs the thread tens of clocks of
// latency, which the tensor pipe would spend idle).
template <int Lead, bool First>
__device__ __forceinline__ void issue_kstep(const uint32_t (&d)[kLevels], const uint32_t (&idesc)[kLevels],
                                            const uint64_t (&ad)[kSlices], const uint64_t (&bd)[kSlicesA]) {
#pragma unroll
    for (int i = 0; i < kIssue; ++i) {
        const int t = kIssueT[i], tp = kIssueTp[i];
        if (t < Lead) continue;
        const int lv = t == 8 ? kLevels - 1 : t + tp - 2;
        mma_f16(d[lv], ad[tp - 1], bd[t - 1], idesc[lv], (First && t == 1) ? 0u : 1u);
    }
}

// The time a tile takes, estimated from its sub-block (in clocks, roughly):
// the MMA phase (each MMA moves its 128 x 16 basis slice and its N x 16
// coefficient slice at ~128 B per clock, about twice that in the loaded
// kernel) and, after it, the epilogue (~3.6 K clocks per 16-column chunk of
// rows some level below 7 reaches, ~0.6 K per chunk of the others, ~1.5 K
// to finish). Only the relative costs matter: they split the tile list into
// per-CTA ranges of equal estimated time.
template <bool Chunked>
__device__ uint32_t tile_cost(const SplitPlan& plan, uint32_t key) {
    const TileSource src = tile_source<Chunked>(plan, key);
    const uint64_t packed = __ldg(src.rows);
    const int npass = pass_geom(packed, 0).npass;
    uint32_t cost = 0;
    for (int pass = 0; pass < npass; ++pass) {
        const PassGeom g = pass_geom(packed, pass);
        uint32_t mma = 0, cols = 0;
        for (int ks = 0; ks < src.ksteps; ++ks) {
            const int lead = step_lead(src.leads, ks);
            for (int i = 0; i < kIssue; ++i) {
                const int t = kIssueT[i], tp = kIssueTp[i];
                if (t < lead) continue;
                const int lv = t == 8 ? kLevels - 1 : t + tp - 2;
                ++mma;
                cols += static_cast<uint32_t>(g.n[lv]);
            }
        }
        const int head = min(g.n[kLevels - 3], g.cols) / 16;
        const int tail = (g.cols - min(g.n[kLevels - 3], g.cols)) / 16;
        cost += 2u * (32u * mma + cols / 4u) + 3600u * head + 580u * tail + 1500u;
    }
    return cost;
}

// Each sub-block's estimated tile time, once per sliced branch (`plan` holds
// that branch alone as its one segment). Tables cut into sub-blocks (degrees
// above 128) get one cost for all: measured at 12x12 / degree 192 / order 14
// (tiles of ~31 lookups, whose time the estimate, made for full tiles, does
// not follow), ranges of equal tile count took 73.0 ms against 74.6-75.4 ms
// with the estimate.
template <bool Chunked>
__global__ void __launch_bounds__(256) split_key_costs(const SplitPlan plan, uint32_t* __restrict__ costs) {
    const uint32_t key = blockIdx.x * blockDim.x + threadIdx.x;
    if (key < plan.nblocks) costs[key] = Chunked ? 1u : tile_cost<Chunked>(plan, key);
}

// The tile list and the per-CTA tile ranges, one thread per key (sub-block).
// Each key's lookups go into tiles of up to 128. CTA b of the assembly takes
// the tiles ranges[b] .. ranges[b + 1] of the block-sorted list, a
// contiguous part of (nearly) equal estimated time: a tile weighs its key's
// cost plus the mean cost (half the tile count's share, half the estimate's:
// measured, that balances the CTAs better than either alone). With C(t) the
// weight of the tiles before tile t and T the total, CTA b starts at the
// first tile with C(t) >= thr(b) = ceil(T * b / ctas). Key q's tiles cover
// the weights [P(q), P(q + 1)) with P(q) = cost_prefix[q] + mean *
// tile_offsets[q], so the key writes the starts of the CTAs whose thr falls
// there; thread 0 writes the CTAs past the last tile (and ranges[ctas]).
__global__ void __launch_bounds__(256) split_tiles(const SplitPlan plan, const uint32_t* __restrict__ counts,
                                                   const uint32_t* __restrict__ offsets,
                                                   const uint32_t* __restrict__ tile_offsets,
                                                   const unsigned long long* __restrict__ cost_prefix,
                                                   const uint32_t* __restrict__ totals, int ctas,
                                                   SplitTile* __restrict__ tiles, uint32_t* __restrict__ ranges) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t ntiles = totals[1];
    const unsigned long long n = static_cast<unsigned long long>(ctas);
    if (ntiles == 0) {
        if (b <= static_cast<uint32_t>(ctas)) ranges[b] = 0;
        return;
    }
    const unsigned long long raw = *reinterpret_cast<const unsigned long long*>(totals + 2);
    const unsigned long long mean = raw / ntiles, total = raw + mean * ntiles;
    if (b == 0)
        for (unsigned long long c = (total - 1) * n / total + 1; c <= n; ++c) ranges[c] = ntiles;
    if (b >= plan.nblocks) return;
    const uint32_t cnt = counts[b];
    if (cnt == 0) return;
    uint32_t t = tile_offsets[b];
    for (uint32_t s = 0; s < cnt; s += kTileN, ++t) tiles[t] = SplitTile{b, offsets[b] + s, min(kTileN * 1u, cnt - s), 0};
    const uint32_t m = (cnt + kTileN - 1) / kTileN;
    const unsigned long long wq = key_cost(plan, b) + mean;
    const unsigned long long p0 = cost_prefix[b] + mean * tile_offsets[b], p1 = p0 + m * wq;
    // CTAs c with p0 <= ceil(T * c / n) < p1
    const unsigned long long c_lo = p0 == 0 ? 0 : (p0 - 1) * n / total + 1;
    const unsigned long long c_hi = min((p1 - 1) * n / total, n - 1);
    for (unsigned long long c = c_lo; c <= c_hi; ++c) {
        const unsigned long long thr = (total * c + n - 1) / n;
        const unsigned long long j = thr > p0 ? (thr - p0 + wq - 1) / wq : 0;
        ranges[c] = tile_offsets[b] + static_cast<uint32_t>(j);
    }
}

template <bool Chunked>
__global__ void __launch_bounds__(kAssemblyThreads, 1) split_assembly(const __grid_constant__ Problem p,
                                                                      const __grid_constant__ Scratch w,
                                                                      const __grid_constant__ SplitPlan plan,
                                                                      const SortedLookup* __restrict__ sorted,
                                                                      const SplitTile* __restrict__ tiles,
                                                                      const uint32_t* __restrict__ totals,
                                                                      int64_t* __restrict__ parts,
                                                                      int32_t* __restrict__ error_flag,
                                                                      unsigned long long* __restrict__ counters,
                                                                      const uint32_t* __restrict__ ranges) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    SplitShared& sh = *reinterpret_cast<SplitShared*>(smem_raw);
    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;
    // each CTA takes a contiguous range of the block-sorted tile list (so the
    // later tiles of a coefficient block find its slices in L2), the ranges
    // of equal estimated time (split_tiles writes them)
    const uint32_t tile_begin = ranges[blockIdx.x];
    const uint32_t tile_end = max(tile_begin, ranges[blockIdx.x + 1]);

    if (tid == 0) {
        for (int i = 0; i < kCStages; ++i) {
            mbar_init(&sh.c_full[i], 1);
            mbar_init(&sh.c_empty[i], 1);
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
        mbar_init(&sh.acc_empty, kEpilogueWarps * 32);
        mbar_init(&sh.drain, 1);
        sh.error = 0;
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == kWarpMma) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(&sh.tmem_base)),
                     "n"(kTmemColumns));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = sh.tmem_base;

    if (warp < kProducerWarps) {
        // ---------------------------------------------- basis producers --
        const int l = tid;  // the lookup of this thread
        uint32_t b_cnt = 0, tile_cnt = 0;
        for (uint32_t tile = tile_begin; tile < tile_end && !failed(sh); ++tile, ++tile_cnt) {
            const SplitTile tl = tiles[tile];
            const int mb = static_cast<int>(tile_cnt % kMetaBufs);
            if (tile_cnt >= kMetaBufs && !mbar_wait(&sh.meta_empty[mb], ((tile_cnt / kMetaBufs) - 1) & 1)) {
                sh.error = 1;
                break;
            }
            const TileSource src = tile_source<Chunked>(plan, tl.block);
            const uint64_t rows = __ldg(reinterpret_cast<const unsigned long long*>(src.rows));
            const bool live = static_cast<uint32_t>(l) < tl.count;
            SortedLookup look{0.0, 0.0, ~uint64_t{0}, 0};
            if (live) look = sorted[tl.start + l];
            const double v = look.v;
            sh.meta[mb].u[l] = look.u;
            sh.meta[mb].info[l] = look.info;
            if (l == 0) {
                sh.meta[mb].count = tl.count;
                sh.meta[mb].exponent = __ldg(src.exponent);
                sh.meta[mb].sub = src.sub;
                sh.meta[mb].rows = rows;
            }
            mbar_arrive(&sh.meta_full[mb]);
            const int npass = pass_geom(rows, 0).npass;
            const int ks_tail = tail_kstep(src.leads, src.ksteps);
            const int64_t vfix = fixed_from_double(v, 62);
            const int b0 = src.kc * kSubK;
            bool ok = true;
            for (int pass = 0; pass < npass && ok; ++pass) {
                // T_b(v) by eight chains of stride 8 (chain j: b = j, j + 8,
                // ...), from T_0..T_8 by the stride-1 recurrence; Q30 from
                // the tail K step on
                ChebChain ch[8];
                int64_t w8;
                {
                    int64_t t8[9];
                    cheb_table8(vfix, t8);
#pragma unroll
                    for (int j = 0; j < 8; ++j) ch[j] = ChebChain{t8[8 - j], t8[j]};
                    w8 = t8[8];
                }
                for (int k = 0; k < b0 / 8; ++k)  // to degrees b0 + j
#pragma unroll
                    for (int j = 0; j < 8; ++j) ch[j].next(w8);
                // one K step's digits (biased Q56 values of b = b0 + 16 ks + m:
                // k = 0..7 hold the even m, k = 8..15 the odd m) into a stage
                auto emit = [&](int ks, const uint64_t (&ye)[8], const uint64_t (&yo)[8]) -> bool {
                    const int sb = static_cast<int>(b_cnt % kBStages);
                    if (b_cnt >= kBStages && !mbar_wait(&sh.b_empty[sb], ((b_cnt / kBStages) - 1) & 1)) {
                        sh.error = 1;
                        return false;
                    }
                    // only the basis slices the K step's MMAs read: t' <= 8 - lead
                    const int tmax = max(1, kSlicesA - step_lead(src.leads, ks));
                    uint16_t* base = sh.basis_ring[sb] + core_offset(l, 0);
#pragma unroll
                    for (int t = 1; t <= kSlices; ++t) {
                        if (t > tmax) break;
                        const uint32_t addr = smem_addr(base + (t - 1) * kTileN * kKStep);
                        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr),
                                     "r"(digit_pair(ye[0], ye[1], t)), "r"(digit_pair(ye[2], ye[3], t)),
                                     "r"(digit_pair(ye[4], ye[5], t)), "r"(digit_pair(ye[6], ye[7], t))
                                     : "memory");
                        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr + 128),
                                     "r"(digit_pair(yo[0], yo[1], t)), "r"(digit_pair(yo[2], yo[3], t)),
                                     "r"(digit_pair(yo[4], yo[5], t)), "r"(digit_pair(yo[6], yo[7], t))
                                     : "memory");
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    mbar_arrive(&sh.b_full[sb]);
                    ++b_cnt;
                    return true;
                };
                int ks = 0;
                for (; ks < ks_tail && ok; ++ks) {  // Q62: all seven digits
                    uint64_t ye[8], yo[8];
                    const int bs = b0 + ks * kKStep;
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const int64_t first = ch[j].next(w8), second = ch[j].next(w8);
                        const uint64_t y1 = static_cast<uint64_t>(bs + j < p.s.nv ? (first + 32) >> 6 : 0) + kDigitBias;
                        const uint64_t y2 =
                            static_cast<uint64_t>(bs + 8 + j < p.s.nv ? (second + 32) >> 6 : 0) + kDigitBias;
                        if (j & 1) {
                            yo[j >> 1] = y1;
                            yo[(j >> 1) + 4] = y2;
                        } else {
                            ye[j >> 1] = y1;
                            ye[(j >> 1) + 4] = y2;
                        }
                    }
                    ok = emit(ks, ye, yo);
                }
                if (ks < src.ksteps && ok) {  // Q30 from the tail K step on: digits 1 and 2
                    ChebChain30 c30[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) c30[j] = ChebChain30{q62_to_q30(ch[j].prev), q62_to_q30(ch[j].cur)};
                    const int32_t w30 = q62_to_q30(w8);
                    for (; ks < src.ksteps && ok; ++ks) {
                        uint64_t ye[8], yo[8];
                        const int bs = b0 + ks * kKStep;
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const int32_t first = c30[j].next(w30), second = c30[j].next(w30);
                            const uint64_t y1 =
                                (bs + j < p.s.nv ? static_cast<uint64_t>(static_cast<int64_t>(first) << 26) : 0) +
                                kDigitBias;
                            const uint64_t y2 =
                                (bs + 8 + j < p.s.nv ? static_cast<uint64_t>(static_cast<int64_t>(second) << 26) : 0) +
                                kDigitBias;
                            if (j & 1) {
                                yo[j >> 1] = y1;
                                yo[(j >> 1) + 4] = y2;
                            } else {
                                ye[j >> 1] = y1;
                                ye[(j >> 1) + 4] = y2;
                            }
                        }
                        ok = emit(ks, ye, yo);
                    }
                }
            }
            if (!ok) break;
        }
    } else if (warp < kProducerWarps + kEpilogueWarps) {
        // ------------------------------------------------------ epilogue --
        const int e = tid - kProducerWarps * 32;  // 0..255
        const int group = e >> 7;                 // columns 4 group + (0..3, 8..11) of every 16
        const int l = e & (kTileN - 1);           // TMEM lane = lookup (warp w reads lanes 32 (w & 3)..)
        const uint32_t lane_base = tmem + (static_cast<uint32_t>((warp & 3) * 32) << 16);
        const int nmax = p.max_order;
        uint32_t tile_cnt = 0, pass_cnt = 0;
        for (uint32_t tile = tile_begin; tile < tile_end; ++tile, ++tile_cnt) {
            const int mb = static_cast<int>(tile_cnt % kMetaBufs);
            const bool meta_ok = mbar_wait(&sh.meta_full[mb], (tile_cnt / kMetaBufs) & 1);
            // (also: the previous tile's second-group sums have been read)
            if (epilogue_any(!meta_ok || failed(sh))) {
                sh.error = 1;
                break;
            }
            const TileMeta& meta = sh.meta[mb];
            const uint64_t rows = meta.rows;
            const int a_sub = Chunked ? (meta.sub / plan.nkc) * kRows : 0;  // first row of the sub-block
            const int64_t ufix = fixed_from_double(meta.u[l], 62);
            uint64_t slo = 0;  // 128-bit sum over the rows some level below 7 reaches
            int64_t shi = 0;
            int64_t tail = 0;  // 64-bit sum over the rows only levels 7 and 8 reach
            const int npass = pass_geom(rows, 0).npass;
            bool ok = true;
            for (int pass = 0; pass < npass; ++pass, ++pass_cnt) {
                const PassGeom g = pass_geom(rows, pass);
                // T_a(u) by four chains of stride 8 (chain q: a = 4 group + q,
                // + 8, ...), from T_0..T_8 by the stride-1 recurrence
                ChebChain ch[4];
                int64_t w8;
                {
                    int64_t t8[9];
                    cheb_table8(ufix, t8);
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        ch[q] = group ? ChebChain{t8[4 - q], t8[4 + q]} : ChebChain{t8[8 - q], t8[q]};
                    w8 = t8[8];
                }
                for (int k = 0; k < (a_sub + g.row0) / 8; ++k)  // to the pass's first row
#pragma unroll
                    for (int q = 0; q < 4; ++q) ch[q].next(w8);
                // the chunks from c_tail on hold only levels 7 and 8
                const int c_tail = g.n[kLevels - 3];
                const bool acc_ok = mbar_wait(&sh.acc_full, pass_cnt & 1);
                if (epilogue_any(!acc_ok)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const int c_head = min(c_tail, g.cols);
                for (int c0 = 0; c0 < c_head; c0 += 16) {
                    // this thread's 8 columns c0 + 4 group + (0..3, 8..11):
                    // value q is row a = c0 + 4 group + (q & 3) + 8 (q >> 2).
                    // W * 2^55 = sum_tau L_tau 2^(55 - 8 tau): levels 7 and 8
                    // folded in FP32, levels 2..6 exact integers
                    const uint32_t col = lane_base + c0 + 4 * group;
                    int64_t wfix[8];
                    {  // levels 8, 7 and 6
                        uint32_t v8[8], v7[8], v6[8];
                        tmem_load_4x2(col + g.col[kLevels - 1], v8);
                        const bool has7 = g.n[kLevels - 2] > c0;
                        if (has7) tmem_load_4x2(col + g.col[kLevels - 2], v7);
                        tmem_load_4x2(col + g.col[kLevels - 3], v6);
                        asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const float f7 = has7 ? __uint_as_float(v7[q]) * 0.5f : 0.0f;
                            wfix[q] = __float2int_rn(fmaf(__uint_as_float(v8[q]), 0.001953125f, f7));
                            wfix[q] += static_cast<int64_t>(__float2int_rn(__uint_as_float(v6[q]))) << 7;
                        }
                    }
                    if (g.n[kLevels - 4] > c0) {  // levels 2..5
                        uint32_t v[kLevels - 3][8];
#pragma unroll
                        for (int lv = 0; lv < kLevels - 3; ++lv)
                            if (g.n[lv] > c0) tmem_load_4x2(col + g.col[lv], v[lv]);
                        asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
                        for (int lv = 0; lv < kLevels - 3; ++lv) {
                            if (g.n[lv] <= c0) continue;
                            const int shift = 39 - 8 * lv;  // 2^(55 - 8 tau), tau = lv + 2
#pragma unroll
                            for (int q = 0; q < 8; ++q)
                                wfix[q] += static_cast<int64_t>(__float2int_rn(__uint_as_float(v[lv][q]))) << shift;
                        }
                    }
                    // sum_a T_a(u) W_a: products rounded to 2^-55, summed exactly
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int64_t tf = ch[q & 3].next(w8);
                        const uint64_t plo = static_cast<uint64_t>(wfix[q]) * static_cast<uint64_t>(tf);
                        int64_t phi = __mul64hi(wfix[q], tf);
                        const uint64_t plo2 = plo + (uint64_t{1} << 61);
                        phi += plo2 < plo ? 1 : 0;
                        const int64_t prod = static_cast<int64_t>((static_cast<uint64_t>(phi) << 2) | (plo2 >> 62));
                        const uint64_t nlo = slo + static_cast<uint64_t>(prod);
                        shi += (prod < 0 ? -1 : 0) + (nlo < slo ? 1 : 0);
                        slo = nlo;
                    }
                }
                if (c_head < g.cols) {
                    // the rows only levels 7 and 8 reach: the levels folded in
                    // FP32 (|W| < 2^24 units of 2^-55), T_a(u) in Q30, 32 x 32
                    // products, a 64-bit sum
                    ChebChain30 c30[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) c30[q] = ChebChain30{q62_to_q30(ch[q].prev), q62_to_q30(ch[q].cur)};
                    const int32_t w30 = q62_to_q30(w8);
                    for (int c0 = c_head; c0 < g.cols; c0 += 16) {
                        const uint32_t col = lane_base + c0 + 4 * group;
                        uint32_t v8[8], v7[8];
                        tmem_load_4x2(col + g.col[kLevels - 1], v8);
                        const bool has7 = g.n[kLevels - 2] > c0;
                        if (has7) tmem_load_4x2(col + g.col[kLevels - 2], v7);
                        asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const float f7 = has7 ? __uint_as_float(v7[q]) * 0.5f : 0.0f;
                            const int32_t wf = __float2int_rn(fmaf(__uint_as_float(v8[q]), 0.001953125f, f7));
                            const int32_t t30 = c30[q & 3].next(w30);
                            tail += (static_cast<int64_t>(wf) * t30 + (int64_t{1} << 29)) >> 30;
                        }
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;");
                mbar_arrive(&sh.acc_empty);  // the next pass's MMAs may write the columns
            }
            if (!ok) {
                sh.error = 1;
                break;
            }
            {  // the 64-bit tail sum into the 128-bit sum
                const uint64_t nlo = slo + static_cast<uint64_t>(tail);
                shi += (tail < 0 ? -1 : 0) + (nlo < slo ? 1 : 0);
                slo = nlo;
            }
            // the second group's sums to the first group's threads, which
            // finish: one thread per lookup, so that the few FP64 operations
            // are issued once per lookup. A block of several sub-blocks
            // leaves its exact 128-bit part for the combine kernel instead.
            if (group == 1) {
                sh.sums[l][0] = static_cast<int64_t>(slo);
                sh.sums[l][1] = shi;
            }
            epilogue_any(false);
            if (group == 0 && static_cast<uint32_t>(l) < meta.count) {
                const uint64_t olo = static_cast<uint64_t>(sh.sums[l][0]);
                const uint64_t nlo = slo + olo;
                shi += sh.sums[l][1] + (nlo < slo ? 1 : 0);
                slo = nlo;
                const uint64_t info = meta.info[l];
                if constexpr (!Chunked) {
                    store_green(p, w, info, int128_to_double(shi, slo, meta.exponent - 55));
                } else {
                    const int64_t slot = part_slot(info, plan, nmax, meta.sub);
                    parts[2 * slot] = static_cast<int64_t>(slo);
                    parts[2 * slot + 1] = shi;
                }
            }
            mbar_arrive(&sh.meta_empty[mb]);
        }
    } else if (warp == kWarpCopy) {
        // ----------------------------------------- coefficient streaming --
        if (lane == 0) {
            uint32_t c_cnt = 0;
            unsigned long long streamed = 0;
            bool ok = true;
            for (uint32_t tile = tile_begin; ok && tile < tile_end && !failed(sh); ++tile) {
                const TileSource src = tile_source<Chunked>(plan, tiles[tile].block);
                const uint64_t rows = __ldg(reinterpret_cast<const unsigned long long*>(src.rows));
                const int npass = pass_geom(rows, 0).npass;
                for (int pass = 0; ok && pass < npass; ++pass) {
                    const PassGeom g = pass_geom(rows, pass);
                    for (int ks = 0; ks < src.ksteps; ++ks, ++c_cnt) {
                        const int st = static_cast<int>(c_cnt % kCStages);
                        if (c_cnt >= kCStages && !mbar_wait(&sh.c_empty[st], ((c_cnt / kCStages) - 1) & 1)) {
                            sh.error = 1;
                            ok = false;
                            break;
                        }
                        // slices lead..8 (the ones before the lead are zero), the
                        // pass's rows (at least one 16-row group, so that every
                        // stage completes by a copy)
                        const int lead = step_lead(src.leads, ks);
                        const uint16_t* from = src.a + static_cast<int64_t>(ks) * (kAStageBytes / 2);
                        sh.c_lead[st] = static_cast<uint32_t>(lead);
                        const int cols = max(g.cols, 16);
                        if (g.row0 == 0 && cols == kRows) {  // whole slices: one copy
                            const uint32_t offset = static_cast<uint32_t>(lead - 1) * (kRows * kKStep);
                            const uint32_t bytes = kAStageBytes - offset * 2;
                            mbar_expect_tx(&sh.c_full[st], bytes);
                            bulk_copy_g2s(sh.coeff_ring[st] + offset, from + offset, bytes, &sh.c_full[st]);
                            streamed += bytes;
                        } else {  // each slice's rows row0 .. row0 + cols
                            const uint32_t bytes = static_cast<uint32_t>(cols) * kKStep * 2;
                            mbar_expect_tx(&sh.c_full[st], bytes * static_cast<uint32_t>(kSlicesA + 1 - lead));
                            for (int t = lead; t <= kSlicesA; ++t) {
                                const uint32_t offset = static_cast<uint32_t>(t - 1) * (kRows * kKStep) +
                                                        static_cast<uint32_t>(g.row0) * kKStep;
                                bulk_copy_g2s(sh.coeff_ring[st] + offset, from + offset, bytes, &sh.c_full[st]);
                                streamed += bytes;
                            }
                        }
                    }
                }
            }
            if (counters) atomicAdd(counters + 1, streamed);
            // copies still in flight (only after an error) land before the CTA exits
            for (uint32_t st = 0; st < static_cast<uint32_t>(kCStages); ++st) {
                if (c_cnt <= st) continue;
                const uint32_t last = c_cnt - 1 - (c_cnt - 1 - st) % kCStages;
                if (!mbar_wait(&sh.c_full[st], (last / kCStages) & 1)) sh.error = 1;
            }
        }
    } else if (warp == kWarpMma) {
        // ---------------------------------------------------- MMA issue --
        if (lane == 0) {
            uint32_t c_cnt = 0, b_cnt = 0, pass_cnt = 0;
            unsigned long long mmas = 0;
            bool ok = true, issued = false;
            for (uint32_t tile = tile_begin; ok && tile < tile_end && !failed(sh); ++tile) {
                const TileSource src = tile_source<Chunked>(plan, tiles[tile].block);
                const uint64_t rows = __ldg(reinterpret_cast<const unsigned long long*>(src.rows));
                const int npass = pass_geom(rows, 0).npass;
                for (int pass = 0; ok && pass < npass; ++pass, ++pass_cnt) {
                    const PassGeom g = pass_geom(rows, pass);
                    // the previous pass's accumulators have been drained
                    if (pass_cnt > 0 && !mbar_wait(&sh.acc_empty, (pass_cnt - 1) & 1)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    // per-level accumulator addresses and instruction descriptors
                    // of the pass; a level without columns writes 16 columns of
                    // the sink at the top of tensor memory, which nothing reads
                    uint32_t dcol[kLevels], idesc[kLevels];
#pragma unroll
                    for (int lv = 0; lv < kLevels; ++lv) {
                        dcol[lv] = tmem + static_cast<uint32_t>(g.n[lv] > 0 ? g.col[lv] : kTmemSink);
                        idesc[lv] = mma_idesc(kTileN, g.n[lv] > 0 ? g.n[lv] : 16);
                    }
                    // accumulator columns a K step's MMAs write, by its lead (the
                    // counter of issued tensor work: 2 x 128 x 16 flops per column)
                    uint32_t cols_at_lead[kSlicesA + 1] = {};
#pragma unroll
                    for (int i = 0; i < kIssue; ++i) {
                        const int t = kIssueT[i], tp = kIssueTp[i];
                        const int lv = t == 8 ? kLevels - 1 : t + tp - 2;
#pragma unroll
                        for (int lead = 1; lead <= kSlicesA; ++lead)
                            if (t >= lead) cols_at_lead[lead] += g.n[lv] > 0 ? g.n[lv] : 16;
                    }
                    for (int ks = 0; ks < src.ksteps; ++ks, ++c_cnt, ++b_cnt) {
                        const int sc = static_cast<int>(c_cnt % kCStages);
                        const int sb = static_cast<int>(b_cnt % kBStages);
                        if (!mbar_wait(&sh.c_full[sc], (c_cnt / kCStages) & 1) ||
                            !mbar_wait(&sh.b_full[sb], (b_cnt / kBStages) & 1)) {
                            ok = false;
                            break;
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;");
                        // the stage's lead (1 in a tile's first K step): pairs
                        // with a coefficient slice before it are zero, not issued
                        const int lead = static_cast<int>(*static_cast<volatile uint32_t*>(&sh.c_lead[sc]));
                        // descriptors of every slice of the two stages (rows row0..
                        // of the coefficients), all in registers before the MMAs;
                        // a slice further on is the same descriptor plus its byte
                        // offset / 16 (the 14-bit address field cannot carry:
                        // shared memory < 256 KiB)
                        uint64_t ad[kSlices], bd[kSlicesA];
                        const uint64_t a0 = smem_desc(smem_addr(sh.basis_ring[sb]), 128, 256);
                        const uint64_t b0 = smem_desc(smem_addr(sh.coeff_ring[sc] + g.row0 * kKStep), 128, 256);
#pragma unroll
                        for (int k = 0; k < kSlices; ++k) ad[k] = a0 + k * (kSliceBytes / 16);
#pragma unroll
                        for (int k = 0; k < kSlicesA; ++k) bd[k] = b0 + k * (kSliceBytes / 16);
                        if (ks == 0) {
                            issue_kstep<1, true>(dcol, idesc, ad, bd);
                        } else {
                            switch (lead) {
                                case 1: issue_kstep<1, false>(dcol, idesc, ad, bd); break;
                                case 2: issue_kstep<2, false>(dcol, idesc, ad, bd); break;
                                case 3: issue_kstep<3, false>(dcol, idesc, ad, bd); break;
                                case 4: issue_kstep<4, false>(dcol, idesc, ad, bd); break;
                                case 5: issue_kstep<5, false>(dcol, idesc, ad, bd); break;
                                case 6: issue_kstep<6, false>(dcol, idesc, ad, bd); break;
                                case 7: issue_kstep<7, false>(dcol, idesc, ad, bd); break;
                                default: issue_kstep<8, false>(dcol, idesc, ad, bd); break;
                            }
                        }
                        mmas += cols_at_lead[ks == 0 ? 1 : lead];
                        issued = true;
                        mma_commit(&sh.c_empty[sc]);
                        mma_commit(&sh.b_empty[sb]);
                    }
                    if (!ok) break;
                    mma_commit(&sh.acc_full);
                }
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
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kTmemColumns));
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
        store_green(p, w, rec.info[base], int128_to_double(hi, lo, *tile_source<true>(plan, key).exponent - 55));
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

size_t split_leads_bytes(int nu, int nv, size_t blocks) {
    int nrb, nkc, ksteps_last;
    split_geometry(nu, nv, &nrb, &nkc, &ksteps_last);
    return blocks * nrb * static_cast<size_t>(row_ksteps(nkc, ksteps_last));
}

size_t split_level_rows_bytes(int nu, int nv, size_t blocks) {
    int nrb, nkc, ksteps_last;
    split_geometry(nu, nv, &nrb, &nkc, &ksteps_last);
    return blocks * nrb * nkc * sizeof(uint64_t);
}

cudaError_t launch_slice_table(const double* coeffs, int nu, int nv, size_t blocks, uint16_t* slices,
                               int32_t* exponents, uint8_t* leads, uint64_t* level_rows, uint32_t* key_costs,
                               cudaStream_t stream) {
    if (blocks == 0) return cudaSuccess;
    int nrb, nkc, ksteps_last;
    split_geometry(nu, nv, &nrb, &nkc, &ksteps_last);
    const size_t grid = blocks * nrb * nkc;
    if (grid > 0x7FFFFFFFu) return cudaErrorInvalidValue;
    slice_blocks<<<static_cast<unsigned>(grid), 256, 0, stream>>>(coeffs, nu, nv, nrb, nkc, ksteps_last, slices,
                                                                  exponents, leads, level_rows);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    // the branch alone as a one-segment plan: its sub-blocks' tile costs
    SplitPlan one{};
    one.segments = 1;
    one.segment_base[0] = 0;
    one.segment_base[1] = static_cast<uint32_t>(grid);
    one.slices[0] = slices;
    one.exponents[0] = exponents;
    one.leads[0] = leads;
    one.level_rows[0] = level_rows;
    one.nblocks = static_cast<uint32_t>(grid);
    one.nrb = nrb;
    one.nkc = nkc;
    one.ksteps_last = ksteps_last;
    const unsigned cgrid = static_cast<unsigned>((grid + 255) / 256);
    if (nrb * nkc > 1)
        split_key_costs<true><<<cgrid, 256, 0, stream>>>(one, key_costs);
    else
        split_key_costs<false><<<cgrid, 256, 0, stream>>>(one, key_costs);
    return cudaGetLastError();
}

size_t split_scratch_bytes(int64_t batch, int max_order, const SplitPlan& plan) {
    const size_t nsub = static_cast<size_t>(plan.nrb) * plan.nkc;
    const size_t nrec = static_cast<size_t>(batch) * max_order * max_order * records_per_pair(plan) * nsub;
    size_t total = 0;
    total += nrec * (4 + 8 + 8 + 8);          // unsorted records
    total += nrec * sizeof(SortedLookup);     // sorted records
    total += static_cast<size_t>(plan.nblocks) * 4 * 4;  // counts, offsets, tile offsets, cursors
    total += static_cast<size_t>(plan.nblocks) * 8;      // estimated-time prefix
    total += (nrec / kTileN + plan.nblocks + 1) * sizeof(SplitTile);  // tiles
    if (nsub > 1) total += nrec * 16;         // 128-bit sub-block parts
    total += 32 + kSplitStatusBytes;          // totals, error flag and counters
    total += (1024 + 1) * 4;                  // per-CTA tile ranges (up to 1,024 SMs)
    return total + 18 * 256;
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
    SortedLookup* sorted = static_cast<SortedLookup*>(take(nrec * sizeof(SortedLookup)));
    uint32_t* counts = static_cast<uint32_t*>(take(plan.nblocks * 4u));
    uint32_t* offsets = static_cast<uint32_t*>(take(plan.nblocks * 4u));
    uint32_t* tile_offsets = static_cast<uint32_t*>(take(plan.nblocks * 4u));
    uint32_t* cursors = static_cast<uint32_t*>(take(plan.nblocks * 4u));
    unsigned long long* cost_prefix = static_cast<unsigned long long*>(take(plan.nblocks * 8u));
    SplitTile* tiles = static_cast<SplitTile*>(take((nrec / kTileN + plan.nblocks + 1) * sizeof(SplitTile)));
    int64_t* parts = nsub > 1 ? static_cast<int64_t*>(take(nrec * 16)) : nullptr;
    uint32_t* totals = static_cast<uint32_t*>(take(32));
    uint32_t* ranges = static_cast<uint32_t*>(take((static_cast<size_t>(sm_count) + 1) * 4));
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
    {
        const int64_t per_warp = descriptor_configs_per_warp(p.max_order);
        const int64_t warps = (p.batch + per_warp - 1) / per_warp;
        split_descriptors<<<static_cast<unsigned>((warps + 3) / 4), 128, 0, stream>>>(p, w, plan, rec, counts);
    }
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    split_scan<<<1, 1024, 0, stream>>>(plan, counts, offsets, tile_offsets, cursors, cost_prefix, totals);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    split_scatter<<<static_cast<unsigned>((nrec + 255) / 256), 256, 0, stream>>>(rec, nrec, offsets, cursors,
                                                                                 sorted);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    const uint32_t tile_threads = std::max(plan.nblocks, static_cast<uint32_t>(sm_count) + 1);
    split_tiles<<<(tile_threads + 255) / 256, 256, 0, stream>>>(plan, counts, offsets, tile_offsets, cost_prefix,
                                                                totals, sm_count, tiles, ranges);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    if (events && events->marks[1]) cudaEventRecord(events->marks[1], stream);
    const size_t smem = sizeof(SplitShared);
    auto kernel = nsub > 1 ? split_assembly<true> : split_assembly<false>;
    err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (err != cudaSuccess) return err;
    kernel<<<sm_count, kAssemblyThreads, smem, stream>>>(p, w, plan, sorted, tiles, totals, parts, error_flag,
                                                         counters, ranges);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    if (nsub > 1) {
        split_combine<<<static_cast<unsigned>((pairs + 127) / 128), 128, 0, stream>>>(p, w, plan, rec, parts);
        err = cudaGetLastError();
    }
    return err;
}

}  // namespace cdet
