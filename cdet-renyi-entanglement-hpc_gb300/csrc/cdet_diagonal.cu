// Deterministic order-1 diagonal observable on the GPU
// (diagonal_green_observable.h:121-327), bit-identical to the reference.
//
//   twisted  = -U / (N1 N2) * sum_{alpha in {0,1}} sum_sites I(alpha, site)
//   ordinary = -U / (N1 N2) * sum_sites I(0, site)        (ordinary tables)
//   I = int_0^beta (G_up + a_dn/U)(G_dn + a_up/U) - a_up a_dn / U^2 dtau
//
// evaluated from the lower-branch diagonal blocks: on the diagonal v = 1, so
// the block collapses to a line sum_b C[a][b] over the u degrees, and the
// tau integrals are the closed-form integrals of T_k and T_i T_j over [-1, 1].
// One CTA per (set, replica, site) item forms its two lines (threads over the
// rows, each row summed in the reference's order) and one thread integrates
// them in the reference's order; a final single thread adds the items in the
// reference's loop order (replica, then y, then x). Every FP64 operation is an
// explicit round-to-nearest intrinsic, as in the reference's double build.
#include "cdet_device.cuh"
#include "cdet_kernels.cuh"

namespace cdet {

namespace {

// chebyshev_uniform_integral_weight (diagonal_green_observable.h:57-67)
__device__ __forceinline__ double uniform_weight(int degree) {
    if (degree & 1) return 0.0;
    if (degree == 0) return 2.0;
    const double d = static_cast<double>(degree);
    return ddiv(2.0, dsub(1.0, dmul(d, d)));
}

struct DiagonalArgs {
    const double* lower[4];  // lower-branch coefficients: twisted up, twisted down, ordinary up, ordinary down
    int n1, n2, nu, nv;
    double beta, shift_up, shift_down;
};

// integrate_diagonal_shifted_product_from_tables (:161-180) for one item.
__global__ void __launch_bounds__(128) diagonal_site_terms(const __grid_constant__ DiagonalArgs a,
                                                           double* __restrict__ items) {
    extern __shared__ double line_smem[];
    double* up_line = line_smem;
    double* down_line = up_line + a.nu;
    double* weight = down_line + a.nu;  // [2 nu]
    const int sites = a.n1 * a.n2;
    const int item = blockIdx.x;
    const int set = item < 2 * sites ? 0 : 1;
    const int replica = set == 0 ? item / sites : 0;
    const int rem = set == 0 ? item - replica * sites : item - 2 * sites;
    const int y = rem / a.n1, x = rem - (rem / a.n1) * a.n1;
    // replica_sitepair_index (replica_chebyshev_tables.h:365-382) of (r, r, x, y, x, y)
    const uint64_t sp = ((((static_cast<uint64_t>(replica) * 2 + replica) * a.n1 + x) * a.n2 + y) * a.n1 + x) *
                            static_cast<uint64_t>(a.n2) +
                        y;
    const uint64_t block = static_cast<uint64_t>(a.nu) * a.nv;
    const double* up = a.lower[set * 2] + sp * block;
    const double* down = a.lower[set * 2 + 1] + sp * block;
    // lower_diagonal_line_coefficients (:69-96): rows summed over v in order
    for (int r = threadIdx.x; r < a.nu; r += blockDim.x) {
        double su = 0.0, sd = 0.0;
        for (int b = 0; b < a.nv; ++b) {
            su = dadd(su, up[static_cast<int64_t>(r) * a.nv + b]);
            sd = dadd(sd, down[static_cast<int64_t>(r) * a.nv + b]);
        }
        up_line[r] = su;
        down_line[r] = sd;
    }
    for (int k = threadIdx.x; k < 2 * a.nu; k += blockDim.x) weight[k] = uniform_weight(k);
    __syncthreads();
    if (threadIdx.x != 0) return;
    // integrate_chebyshev_line (:121-130)
    double iu = 0.0, id = 0.0;
    for (int k = 0; k < a.nu; ++k) {
        iu = dadd(iu, dmul(up_line[k], weight[k]));
        id = dadd(id, dmul(down_line[k], weight[k]));
    }
    const double up_integral = ddiv(dmul(a.beta, iu), 2.0);
    const double down_integral = ddiv(dmul(a.beta, id), 2.0);
    // integrate_chebyshev_line_product (:141-159)
    double ip = 0.0;
    for (int i = 0; i < a.nu; ++i) {
        const double lv = up_line[i];
        for (int j = 0; j < a.nu; ++j) {
            const int diff = i > j ? i - j : j - i;
            const double w = ddiv(dadd(weight[i + j], weight[diff]), 2.0);
            ip = dadd(ip, dmul(dmul(lv, down_line[j]), w));
        }
    }
    const double product = ddiv(dmul(a.beta, ip), 2.0);
    items[item] = dadd(dadd(product, dmul(a.shift_up, down_integral)), dmul(a.shift_down, up_integral));
}

// replica_log_partition_first_order_density_typed (:237-273),
// ordinary_log_partition_first_order_density_typed (:275-303) and
// normalized_log_partition_first_order_density_dd (:305-323).
__global__ void diagonal_finish(const double* __restrict__ items, int sites, double n1, double n2, double u,
                                double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double twisted_sum = 0.0, ordinary_sum = 0.0;
    for (int i = 0; i < 2 * sites; ++i) twisted_sum = dadd(twisted_sum, items[i]);
    for (int i = 0; i < sites; ++i) ordinary_sum = dadd(ordinary_sum, items[2 * sites + i]);
    const double denom = dmul(n1, n2);
    const double twisted = ddiv(dmul(-u, twisted_sum), denom);
    const double ordinary = ddiv(dmul(-u, ordinary_sum), denom);
    out[0] = dsub(twisted, dmul(2.0, ordinary));
    out[1] = twisted;
    out[2] = ordinary;
}

}  // namespace

cudaError_t launch_diagonal_order1(const TableDev* const tables[4], int n1, int n2, int nu, int nv, double beta,
                                   double u, double alpha_up, double alpha_down, double* items, double* out,
                                   cudaStream_t stream) {
    DiagonalArgs a{};
    for (int k = 0; k < 4; ++k) a.lower[k] = tables[k]->lower;
    a.n1 = n1;
    a.n2 = n2;
    a.nu = nu;
    a.nv = nv;
    a.beta = beta;
    // diagonal_up_shift = alpha_down / U, diagonal_down_shift = alpha_up / U, in double (:255-256)
    a.shift_up = alpha_down / u;
    a.shift_down = alpha_up / u;
    const int sites = n1 * n2;
    const size_t smem = static_cast<size_t>(4 * nu) * sizeof(double);
    diagonal_site_terms<<<3 * sites, 128, smem, stream>>>(a, items);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    diagonal_finish<<<1, 32, 0, stream>>>(items, sites, static_cast<double>(n1), static_cast<double>(n2), u, out);
    return cudaGetLastError();
}

}  // namespace cdet
