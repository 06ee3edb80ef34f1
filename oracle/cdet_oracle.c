/*
 * CPU restatement of the reference CDet Renyi-2 integrand (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY (see cdet_oracle.h). Each function cites the
 * reference file:line it restates; all paths are relative to the reference
 * project (Boyuan-Shi-0607/cdet-renyi-entanglement-hpc). Compile with
 * -ffp-contract=off: the operation order below is the reference's, and every
 * multiply and add must round separately, exactly as on an x86-64 build.
 */
#include "cdet_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_BAD_INPUT 4
#define ORACLE_MAX_ORDER 24

/* ---------------------------------------------------------------- layout --- */

/* replica_sitepair_index (replica_chebyshev_tables.h:365-382). */
static uint64_t sitepair_index(int ra, int rb, int x1, int y1, int x2, int y2, int n1, int n2) {
    return (((((uint64_t)ra * 2u + (uint64_t)rb) * (uint64_t)n1 + (uint64_t)x1) * (uint64_t)n2 +
             (uint64_t)y1) * (uint64_t)n1 + (uint64_t)x2) * (uint64_t)n2 + (uint64_t)y2;
}

static double clamp_unit(double value) {
    /* clamp_to_unit_interval (g_funcs.h:300-309) */
    if (value < -1.0) return -1.0;
    if (value > 1.0) return 1.0;
    return value;
}

/* prepare_green_lookup_descriptor (g_funcs.h:609-653). The returned index is
 * the corner index on the corner path and the coefficient block base
 * (sitepair * nu * nv) otherwise. */
int oracle_lookup_descriptor(int ra, int rb, double tau1, double tau2, int x1, int y1, int x2,
                             int y2, double beta, double branch_eps, int nu, int nv, int n1,
                             int n2, int upper, int* use_corner, uint64_t* index, double* u,
                             double* v) {
    const uint64_t sp = sitepair_index(ra, rb, x1, y1, x2, y2, n1, n2);
    *u = 0.0;
    *v = 0.0;
    if (upper) {
        if (tau1 < branch_eps) {
            *use_corner = 1;
            *index = sp;
            return 0;
        }
        *u = clamp_unit(2.0 * tau1 / beta - 1.0);
        *v = clamp_unit(2.0 * tau2 / tau1 - 1.0);
    } else {
        if (tau2 < branch_eps) {
            *use_corner = 1;
            *index = sp;
            return 0;
        }
        *u = clamp_unit(2.0 * tau2 / beta - 1.0);
        *v = clamp_unit(2.0 * tau1 / tau2 - 1.0);
    }
    *use_corner = 0;
    *index = sp * (uint64_t)nu * (uint64_t)nv;
    return 0;
}

/* clenshaw_from_contiguous_coeffs / clenshaw_pair_from_contiguous_coeffs
 * (g_funcs.h:395-463): sum_{k<=degree} c[k] T_k(x). */
static double clenshaw(const double* c, int degree, double x) {
    if (degree < 0) return 0.0;
    if (degree == 0) return c[0];
    if (degree == 1) return c[0] + c[1] * x;
    const double two_x = 2.0 * x;
    double b1 = 0.0, b2 = 0.0;
    for (int k = degree; k >= 1; --k) {
        const double bk = c[k] + two_x * b1 - b2;
        b2 = b1;
        b1 = bk;
    }
    return c[0] + b1 * x - b2;
}

/* chebyshev_sum_2d_pair_from_ptrs (g_funcs.h:687-763): a Clenshaw sum along v
 * on every row of the nu x nv block (row-major, v fastest), then one along u
 * over the row values. The fixed-degree specialisations (:561-578) perform
 * the same operations in the same order. */
static double chebyshev_2d(const double* block, double u, double v, int nu, int nv) {
    double rows[512];
    for (int a = 0; a < nu; ++a) rows[a] = clenshaw(block + (size_t)a * (size_t)nv, nv - 1, v);
    return clenshaw(rows, nu - 1, u);
}

/* evaluate_green_pair_descriptor (g_funcs.h:793-818). */
void oracle_green_pair(const oracle_table* up, const oracle_table* down, int upper,
                       int use_corner, uint64_t index, double u, double v, int nu, int nv,
                       double* up_value, double* down_value) {
    if (use_corner) {
        *up_value = upper ? up->upper_corners[index] : up->lower_corners[index];
        *down_value = upper ? down->upper_corners[index] : down->lower_corners[index];
        return;
    }
    const double* cu = (upper ? up->upper_coeffs : up->lower_coeffs) + index;
    const double* cd = (upper ? down->upper_coeffs : down->lower_coeffs) + index;
    *up_value = chebyshev_2d(cu, u, v, nu, nv);
    *down_value = chebyshev_2d(cd, u, v, nu, nv);
}

/* ---------------------------------------------------------- vertex decode --- */

typedef struct vertex {
    double tau, tau_unit;
    int x, y, replica;
} vertex;

/* sampled_coordinate_to_index (g_funcs.h:315-342): floor then clamp to
 * [0, extent-1]. The reference throws std::overflow_error outside the int
 * range; non-finite input is undefined there. Both are reported here. */
static int coordinate_to_index(double coordinate, int extent, int* bad) {
    if (!isfinite(coordinate) || coordinate <= -2147483648.0 || coordinate >= 2147483648.0) {
        *bad = 1;
        return 0;
    }
    int index = (int)floor(coordinate);
    if (index < 0) index = 0;
    if (index >= extent) index = extent - 1;
    return index;
}

/* Vertex decode of integrand_temp_typed (integrand_replica_randomly_sampled.h:422-432)
 * with sampled_replica_from_unit_coordinate_typed (:142-153). */
static int decode_vertices(const oracle_scalars* s, const double* args, int order,
                           int replica_count, vertex* out) {
    int bad = 0;
    for (int i = 0; i < order; ++i) {
        const double* a = args + 4 * i;
        if (!isfinite(a[0])) bad = 1;
        out[i].tau_unit = a[0];
        out[i].tau = s->beta * a[0];
        out[i].x = coordinate_to_index((double)s->n1 * a[1], s->n1, &bad);
        out[i].y = coordinate_to_index((double)s->n2 * a[2], s->n2, &bad);
        if (replica_count <= 1) {
            out[i].replica = 0;
        } else {
            int r = coordinate_to_index((double)replica_count * a[3], replica_count, &bad);
            out[i].replica = r < 0 ? 0 : (r > replica_count - 1 ? replica_count - 1 : r);
        }
    }
    return bad;
}

/* Green-matrix fill of integrand_temp_typed (:434-484) and of the all-subset
 * variant (:698-776): entry (i,j) of each spin matrix is the table value at
 * (vertex i, vertex j), the diagonal gets the crossed alpha shift, and every
 * entry is multiplied by sqrt(U*N1*N2*beta). diag_up/diag_down (optional)
 * receive the shifted, unscaled diagonal the all-subset singletons use. */
static void fill_from_vertices(const oracle_scalars* s, const oracle_table* tu,
                               const oracle_table* td, const vertex* vx, int order,
                               double* mat_up, double* mat_down, double* diag_up,
                               double* diag_down) {
    for (int idx = 0; idx < order * order; ++idx) {
        const int i = idx / order;
        const int j = idx - i * order;
        const int upper = (i != j) && (vx[i].tau_unit > vx[j].tau_unit);
        int corner;
        uint64_t index;
        double u, v, up, down;
        oracle_lookup_descriptor(vx[i].replica, vx[j].replica, vx[i].tau, vx[j].tau, vx[i].x,
                                 vx[i].y, vx[j].x, vx[j].y, s->beta, s->branch_eps, s->cheb_nu,
                                 s->cheb_nv, s->n1, s->n2, upper, &corner, &index, &u, &v);
        oracle_green_pair(tu, td, upper, corner, index, u, v, s->cheb_nu, s->cheb_nv, &up, &down);
        if (i == j) {
            if (diag_up) diag_up[i] = up + s->diag_up_shift;
            if (diag_down) diag_down[i] = down + s->diag_down_shift;
            up += s->diag_up_shift;
            down += s->diag_down_shift;
        }
        mat_up[idx] = up * s->scale;
        mat_down[idx] = down * s->scale;
    }
}

int oracle_fill_green(const oracle_scalars* s, const oracle_table* up, const oracle_table* down,
                      const double* unit_vertices, int order, int replica_count, double* mat_up,
                      double* mat_down, double* diag_up, double* diag_down) {
    vertex vx[ORACLE_MAX_ORDER];
    if (order < 1 || order > ORACLE_MAX_ORDER) return ORACLE_BAD_INPUT;
    if (decode_vertices(s, unit_vertices, order, replica_count, vx)) return ORACLE_BAD_INPUT;
    fill_from_vertices(s, up, down, vx, order, mat_up, mat_down, diag_up, diag_down);
    return 0;
}

/* ------------------------------------------------------ principal minors --- */

/* determinant_principal_minor_from_buffer (fast_principle_minors.h:39-105):
 * partial-pivot LU of the principal submatrix selected by mask. */
static double minor_by_lu(const double* a, int n, uint64_t mask) {
    int idx[64];
    int k = 0;
    for (int i = 0; i < n; ++i)
        if (mask & ((uint64_t)1 << i)) idx[k++] = i;
    if (k == 0) return 1.0;
    double m[ORACLE_MAX_ORDER * ORACLE_MAX_ORDER];
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
        det *= pivot;
        for (int row = col + 1; row < k; ++row) {
            const double factor = m[row * k + col] / pivot;
            if (factor == 0.0) continue;
            m[row * k + col] = 0.0;
            for (int c = col + 1; c < k; ++c) m[row * k + c] = fma(-factor, m[col * k + c], m[row * k + c]);
        }
    }
    return sign < 0 ? -det : det;
}

/* determinant_principal_minors_from_buffer (fast_principle_minors.h:107-115). */
void oracle_minors_by_lu(const double* a, int n, double* pm_out) {
    const uint64_t count = (uint64_t)1 << n;
    for (uint64_t mask = 1; mask < count; ++mask) pm_out[mask - 1] = minor_by_lu(a, n, mask);
}

/* mat2pm_from_buffer (fast_principle_minors.h:120-246): all principal minors
 * of A + pI by a level-by-level Schur-complement recursion, a prefix product,
 * then removal of the uniform shift p by multilinearity. A pivot with
 * |a+p| <= tol*max|A| (or 0) sends the whole matrix to the LU fallback.
 * Returns 1 when the fallback ran, 0 otherwise, -1 on a bad n. */
int oracle_mat2pm(const double* a, int n, double tol, double shift, double* pm_out) {
    if (n <= 0 || n > ORACLE_MAX_ORDER) return -1;
    const uint64_t subset_count = (uint64_t)1 << n;
    const int matrix_size = n * n;
    for (uint64_t i = 0; i + 1 < subset_count; ++i) pm_out[i] = 0.0;

    double max_abs = 0.0;
    for (int i = 0; i < matrix_size; ++i) {
        const double e = fabs(a[i]);
        if (e > max_abs) max_abs = e;
    }
    const int explicit_shift = !(shift < 0.0);
    const double p = explicit_shift ? shift : max_abs / (double)matrix_size;
    if (max_abs == 0.0 && p == 0.0) return 0;
    const double fallback_eps = (tol > 0.0 && max_abs > 0.0) ? tol * max_abs : 0.0;

    size_t list_size = (size_t)matrix_size;
    for (int level = 0; level < n - 1; ++level) {
        const size_t ns = (size_t)(n - level - 1);
        const size_t cand = ((size_t)1 << (level + 1)) * ns * ns;
        if (cand > list_size) list_size = cand;
    }
    double* old_list = (double*)malloc(list_size * sizeof(double));
    double* new_list = (double*)malloc(list_size * sizeof(double));
    double* shifted = (double*)malloc(subset_count * sizeof(double));
    memcpy(old_list, a, (size_t)matrix_size * sizeof(double));
    for (uint64_t i = 0; i < subset_count; ++i) shifted[i] = p;
    shifted[0] = 1.0;
    shifted[1] += old_list[0];

    size_t minor_index = 2;
    int fell_back = 0;
    for (int level = 0; level < n - 1 && !fell_back; ++level) {
        const size_t old_size = (size_t)(n - level);
        const size_t old_msize = old_size * old_size;
        const size_t new_size = old_size - 1;
        const size_t new_msize = new_size * new_size;
        const size_t sets = (size_t)1 << level;
        for (size_t set = 0; set < sets; ++set) {
            size_t dst_without = set * new_msize;
            const size_t src = set * old_msize;
            const size_t first_column = src + old_size;
            size_t dst_with = dst_without + sets * new_msize;
            const double pivot = old_list[src] + p;
            const double pivot_abs = fabs(pivot);
            if (pivot_abs == 0.0 || (fallback_eps > 0.0 && pivot_abs <= fallback_eps)) {
                fell_back = 1;
                break;
            }
            const double inverse = 1.0 / pivot;
            size_t row_start = first_column + 1;
            size_t column_start = first_column;
            for (size_t row = 0; row < new_size; ++row) {
                size_t top_row = src + 1;
                const double factor = old_list[column_start] * inverse;
                for (size_t col = 0; col < new_size; ++col) {
                    const double base = old_list[row_start];
                    new_list[dst_without] = base;
                    new_list[dst_with] = fma(-old_list[top_row], factor, base);
                    ++top_row;
                    ++row_start;
                    ++dst_without;
                    ++dst_with;
                }
                ++row_start;
                column_start += old_size;
            }
        }
        if (fell_back) break;
        for (size_t m = 0; m < 2 * sets; ++m) shifted[minor_index++] += new_list[m * new_msize];
        double* t = old_list;
        old_list = new_list;
        new_list = t;
    }
    if (fell_back) {
        free(old_list);
        free(new_list);
        free(shifted);
        oracle_minors_by_lu(a, n, pm_out);
        return 1;
    }

    uint64_t step = 1;
    for (int level = 0; level < n; ++level) {
        for (uint64_t set = step + 1; set < 2 * step; ++set) shifted[set] *= shifted[set - step];
        step <<= 1;
    }
    step = subset_count;
    for (int level = n; level > 0; --level) {
        const uint64_t half = step >> 1;
        for (uint64_t set = step - 1;; --set) {
            for (uint64_t ss = set; ss < subset_count; ss += step)
                shifted[ss] = fma(-p, shifted[ss - half], shifted[ss]);
            if (set == half) break;
        }
        step = half;
    }
    for (uint64_t mask = 1; mask < subset_count; ++mask) pm_out[mask - 1] = shifted[mask];
    free(old_list);
    free(new_list);
    free(shifted);
    return 0;
}

/* ------------------------------------------------------------------ CDet --- */

static int popcount64(uint64_t x) {
    int c = 0;
    while (x) {
        x &= x - 1;
        ++c;
    }
    return c;
}

/* compute_dp_ztransform (integrand_replica_randomly_sampled.h:226-290): the
 * connected sum of a[m] = up[m-1]*down[m-1] anchored at vertex 0, masks taken
 * in popcount order, with the roundoff filter |acc| < eps0*safety*sum|terms|. */
double oracle_ztransform(const double* up, const double* down, int n, double eps0,
                         double safety) {
    const uint64_t count = (uint64_t)1 << n;
    double* a = (double*)malloc(count * sizeof(double));
    double* dp = (double*)calloc(count, sizeof(double));
    const double threshold = eps0 * safety;
    const int filter = threshold > 0.0;
    a[0] = 0.0;
    for (uint64_t m = 1; m < count; ++m) a[m] = up[m - 1] * down[m - 1];
    for (int i = 0; i < n; ++i) dp[(uint64_t)1 << i] = a[(uint64_t)1 << i];
    for (int bits = 2; bits <= n; ++bits) {
        for (uint64_t mask = 0; mask < count; ++mask) {
            if (popcount64(mask) != bits) continue;
            double acc = a[mask];
            double rhs = fabs(a[mask]);
            if (mask & 1u) {
                for (uint64_t sub = (mask - 1) & mask; sub; sub = (sub - 1) & mask) {
                    if ((sub & 1u) == 0u) continue;
                    const double term = dp[sub] * a[mask ^ sub];
                    acc = acc - term;
                    rhs += fabs(term);
                }
                if (filter && fabs(acc) < threshold * rhs) acc = 0.0;
            }
            dp[mask] = acc;
        }
    }
    const double result = dp[count - 1];
    free(a);
    free(dp);
    return result;
}

/* compute_dp_ztransform_all_subsets (:292-347): every mask anchored at its
 * lowest set bit. dp_out has 2^n entries, dp_out[0] = 0. */
void oracle_ztransform_all(const double* up, const double* down, int n, double eps0,
                           double safety, double* dp) {
    const uint64_t count = (uint64_t)1 << n;
    double* a = (double*)calloc(count, sizeof(double));
    const double threshold = eps0 * safety;
    const int filter = threshold > 0.0;
    for (uint64_t m = 0; m < count; ++m) dp[m] = 0.0;
    for (uint64_t m = 1; m < count; ++m) a[m] = up[m - 1] * down[m - 1];
    for (int i = 0; i < n; ++i) dp[(uint64_t)1 << i] = a[(uint64_t)1 << i];
    for (int bits = 2; bits <= n; ++bits) {
        for (uint64_t mask = 0; mask < count; ++mask) {
            if (popcount64(mask) != bits) continue;
            const uint64_t anchor = mask & (~mask + 1);
            double acc = a[mask];
            double rhs = fabs(a[mask]);
            for (uint64_t sub = (mask - 1) & mask; sub; sub = (sub - 1) & mask) {
                if ((sub & anchor) == 0u) continue;
                const double term = dp[sub] * a[mask ^ sub];
                acc = acc - term;
                rhs += fabs(term);
            }
            if (filter && fabs(acc) < threshold * rhs) acc = 0.0;
            dp[mask] = acc;
        }
    }
    free(a);
}

/* ----------------------------------------------------------- double-double --- */

/* DoubleDouble arithmetic (utility/types.h:30-182): Dekker/Knuth error-free
 * transforms in the arrangement the reference uses. */
typedef struct dd {
    double hi, lo;
} dd;

static double two_sum(double a, double b, double* err) {
    const double s = a + b;
    const double bb = s - a;
    *err = (a - (s - bb)) + (b - bb);
    return s;
}
static double quick_two_sum(double a, double b, double* err) {
    const double s = a + b;
    *err = b - (s - a);
    return s;
}
static double two_prod(double a, double b, double* err) {
    const double p = a * b;
    *err = fma(a, b, -p);
    return p;
}
static dd dd_make(double hi, double lo) {
    dd r = {hi, lo};
    return r;
}
static dd dd_add(dd x, dd y) {
    double s2, t2;
    double s1 = two_sum(x.hi, y.hi, &s2);
    const double t1 = two_sum(x.lo, y.lo, &t2);
    s2 += t1;
    s1 = quick_two_sum(s1, s2, &s2);
    s2 += t2;
    dd r;
    r.hi = quick_two_sum(s1, s2, &r.lo);
    return r;
}
static dd dd_sub(dd x, dd y) { return dd_add(x, dd_make(-y.hi, -y.lo)); }
static dd dd_mul(dd x, dd y) {
    double e;
    const double p = two_prod(x.hi, y.hi, &e);
    e += x.hi * y.lo + x.lo * y.hi + x.lo * y.lo;
    dd r;
    r.hi = quick_two_sum(p, e, &r.lo);
    return r;
}
static dd dd_div(dd x, dd y) {
    const double q1 = x.hi / y.hi;
    const dd r = dd_sub(x, dd_mul(dd_make(q1, 0.0), y));
    const double q2 = (r.hi + r.lo) / y.hi;
    dd q = dd_add(dd_make(q1, 0.0), dd_make(q2, 0.0));
    const double s = q.hi + q.lo;
    q.lo = q.lo - (s - q.hi);
    q.hi = s;
    return q;
}
static int dd_finite(dd x) { return isfinite(x.hi) && isfinite(x.lo); }

/* cdet_order_prefactor<DoubleDouble> (integrand_replica_randomly_sampled.h:155-159):
 * (-r)^n / (n! * N1 * N2). (-r)^n is an exact power (r is 1 or 2). */
void oracle_prefactor_dd(int order, int n1, int n2, int replica_count, double* hi, double* lo) {
    double power = 1.0;
    for (int i = 0; i < order; ++i) power *= -(double)replica_count;
    dd factorial = dd_make(1.0, 0.0);
    for (int i = 1; i <= order; ++i) factorial = dd_mul(factorial, dd_make((double)i, 0.0));
    const dd den = dd_mul(dd_mul(factorial, dd_make((double)n1, 0.0)), dd_make((double)n2, 0.0));
    const dd q = dd_div(dd_make(power, 0.0), den);
    *hi = q.hi;
    *lo = q.lo;
}

/* cdet_order_prefactor<double> (:160-170): long double on the host. */
double oracle_prefactor_ld(int order, int n1, int n2, int replica_count) {
    long double num = 1.0L;
    for (int i = 0; i < order; ++i) num *= -(long double)replica_count;
    long double den = (long double)n1 * (long double)n2;
    for (int i = 2; i <= order; ++i) den *= (long double)i;
    return (double)(num / den);
}

/* ------------------------------------------------------------- integrand --- */

static double order1_raw(const oracle_scalars* s, double shifted_up, double shifted_down,
                         int replica_count) {
    /* order1_density_integrand_from_sampled_vertex (:173-213) and the
     * all-subset singletons (:835-846). */
    const double counterterm = s->diag_up_shift * s->diag_down_shift;
    return (double)(-replica_count) * s->u * s->beta * (shifted_up * shifted_down - counterterm);
}

/* One table set of integrand_temp_typed (:349-547): fill, minors of both
 * spins, anchored CDet, DD prefactor. */
static int integrand_one_set(const oracle_scalars* s, const oracle_table* tu,
                             const oracle_table* td, const double* args, int order,
                             int replica_count, dd* value) {
    vertex vx[ORACLE_MAX_ORDER];
    double mu[ORACLE_MAX_ORDER * ORACLE_MAX_ORDER], md[ORACLE_MAX_ORDER * ORACLE_MAX_ORDER];
    if (decode_vertices(s, args, order, replica_count, vx)) return ORACLE_BAD_INPUT;
    fill_from_vertices(s, tu, td, vx, order, mu, md, NULL, NULL);
    const size_t count = ((size_t)1 << order) - 1;
    double* pu = (double*)malloc(count * sizeof(double));
    double* pd = (double*)malloc(count * sizeof(double));
    int status = 0;
    if (oracle_mat2pm(mu, order, s->tol_fpm, s->fpm_shift, pu) == 1) status |= ORACLE_FPM_FALLBACK;
    if (oracle_mat2pm(md, order, s->tol_fpm, s->fpm_shift, pd) == 1) status |= ORACLE_FPM_FALLBACK;
    const double c = oracle_ztransform(pu, pd, order, s->z_eps0, s->z_safety);
    free(pu);
    free(pd);
    dd pref;
    oracle_prefactor_dd(order, s->n1, s->n2, replica_count, &pref.hi, &pref.lo);
    *value = dd_mul(pref, dd_make(c, 0.0));
    if (!dd_finite(*value)) status |= ORACLE_NONFINITE;
    return status;
}

/* evaluate_cdet_density_integrand_double (cdet_integrand_evaluator.h:542-560)
 * through evaluate_cdet_density_integrand_for_real (:233-263) and the
 * order-1 branch (:171-201): twisted (r=2) minus twice ordinary (r=1) in
 * double-double, rounded to double. */
int oracle_integrand(const oracle_scalars* s, const oracle_tables* t, const double* args,
                     int order, double* value) {
    *value = 0.0;
    if (order <= 0 || order > ORACLE_MAX_ORDER) return ORACLE_BAD_INPUT;
    dd twisted, ordinary;
    int status = 0;
    if (order == 1) {
        vertex vx[2];
        double v[2];
        const oracle_table* tabs[2][2] = {{&t->twisted_up, &t->twisted_down},
                                          {&t->ordinary_up, &t->ordinary_down}};
        for (int set = 0; set < 2; ++set) {
            const int r = set == 0 ? 2 : 1;
            if (decode_vertices(s, args, 1, r, vx)) return ORACLE_BAD_INPUT;
            int corner;
            uint64_t index;
            double u, w, up, down;
            oracle_lookup_descriptor(vx[0].replica, vx[0].replica, vx[0].tau, vx[0].tau, vx[0].x,
                                     vx[0].y, vx[0].x, vx[0].y, s->beta, s->branch_eps,
                                     s->cheb_nu, s->cheb_nv, s->n1, s->n2, 0, &corner, &index,
                                     &u, &w);
            oracle_green_pair(tabs[set][0], tabs[set][1], 0, corner, index, u, w, s->cheb_nu,
                              s->cheb_nv, &up, &down);
            v[set] = order1_raw(s, up + s->diag_up_shift, down + s->diag_down_shift, r);
        }
        twisted = dd_make(v[0], 0.0);
        ordinary = dd_make(v[1], 0.0);
    } else {
        status |= integrand_one_set(s, &t->twisted_up, &t->twisted_down, args, order, 2, &twisted);
        status |= integrand_one_set(s, &t->ordinary_up, &t->ordinary_down, args, order, 1,
                                    &ordinary);
        if (status & ORACLE_BAD_INPUT) return status;
    }
    const dd result = dd_sub(twisted, dd_mul(dd_make(2.0, 0.0), ordinary));
    *value = result.hi + result.lo;
    return status;
}

/* integrand_all_subset_values_typed_into (:549-878) for one table set. */
static int all_subsets_one_set(const oracle_scalars* s, const oracle_table* tu,
                               const oracle_table* td, const double* args, int n,
                               int replica_count, double* values) {
    vertex vx[ORACLE_MAX_ORDER];
    double mu[ORACLE_MAX_ORDER * ORACLE_MAX_ORDER], md[ORACLE_MAX_ORDER * ORACLE_MAX_ORDER];
    double du[ORACLE_MAX_ORDER], ddn[ORACLE_MAX_ORDER];
    if (decode_vertices(s, args, n, replica_count, vx)) return ORACLE_BAD_INPUT;
    fill_from_vertices(s, tu, td, vx, n, mu, md, du, ddn);
    const size_t count = (size_t)1 << n;
    double* pu = (double*)malloc(count * sizeof(double));
    double* pd = (double*)malloc(count * sizeof(double));
    double* dp = (double*)malloc(count * sizeof(double));
    int status = 0;
    if (oracle_mat2pm(mu, n, s->tol_fpm, s->fpm_shift, pu) == 1) status |= ORACLE_FPM_FALLBACK;
    if (oracle_mat2pm(md, n, s->tol_fpm, s->fpm_shift, pd) == 1) status |= ORACLE_FPM_FALLBACK;
    oracle_ztransform_all(pu, pd, n, s->z_eps0, s->z_safety, dp);
    values[0] = 0.0;
    for (int i = 0; i < n; ++i) {
        const double v = order1_raw(s, du[i], ddn[i], replica_count);
        if (!isfinite(v)) status |= ORACLE_NONFINITE;
        values[(size_t)1 << i] = v;
    }
    double pref[ORACLE_MAX_ORDER + 1];
    for (int k = 2; k <= n; ++k) pref[k] = oracle_prefactor_ld(k, s->n1, s->n2, replica_count);
    for (size_t mask = 1; mask < count; ++mask) {
        const int k = popcount64(mask);
        if (k <= 1) continue;
        const double v = pref[k] * dp[mask];
        if (!isfinite(v)) status |= ORACLE_NONFINITE;
        values[mask] = v;
    }
    free(pu);
    free(pd);
    free(dp);
    return status;
}

/* evaluate_cdet_density_all_subset_integrands_double_into
 * (cdet_integrand_evaluator.h:562-583, :304-351): twisted values minus twice
 * the ordinary values, mask by mask, in double. */
int oracle_all_subsets(const oracle_scalars* s, const oracle_tables* t, const double* args,
                       int n, double* values) {
    if (n <= 1 || n > ORACLE_MAX_ORDER) return ORACLE_BAD_INPUT;
    const size_t count = (size_t)1 << n;
    double* ordinary = (double*)malloc(count * sizeof(double));
    int status = all_subsets_one_set(s, &t->twisted_up, &t->twisted_down, args, n, 2, values);
    status |= all_subsets_one_set(s, &t->ordinary_up, &t->ordinary_down, args, n, 1, ordinary);
    if (!(status & ORACLE_BAD_INPUT))
        for (size_t m = 0; m < count; ++m) values[m] -= 2.0 * ordinary[m];
    free(ordinary);
    return status;
}

/* ------------------------------------------------- long double truth --- */
/* A higher-precision evaluation of the same integrand for error studies, the
 * role the reference gives its INTEGRAND_REAL=double_double /
 * VECTOR_REAL=long_double mode (precision_config.h:15-26): the same decoded
 * vertices and the same double (u, v) as the FP64 form, then the Chebyshev
 * sums, the diagonal shifts and the scale, every principal minor (a
 * partial-pivot LU of each principal submatrix), the anchored connected
 * recursion without the round-off filter and the prefactor, all in long
 * double (64-bit significand on x86-64, 113-bit on AArch64). It follows no
 * reference operation order and is compared with nothing bit for bit: it is
 * the value the FP64 and split forms approximate. */
static long double clenshaw_ld(const double* c, int degree, long double x) {
    if (degree < 0) return 0.0L;
    if (degree == 0) return (long double)c[0];
    const long double two_x = 2.0L * x;
    long double b1 = 0.0L, b2 = 0.0L;
    for (int k = degree; k >= 1; --k) {
        const long double bk = (long double)c[k] + two_x * b1 - b2;
        b2 = b1;
        b1 = bk;
    }
    return (long double)c[0] + b1 * x - b2;
}

static long double chebyshev_2d_ld(const double* block, double u, double v, int nu, int nv) {
    long double rows[512];
    for (int a = 0; a < nu; ++a) rows[a] = clenshaw_ld(block + (size_t)a * (size_t)nv, nv - 1, (long double)v);
    /* the outer sum over rows, on long double row values */
    if (nu == 1) return rows[0];
    const long double x = (long double)u, two_x = 2.0L * x;
    long double b1 = 0.0L, b2 = 0.0L;
    for (int k = nu - 1; k >= 1; --k) {
        const long double bk = rows[k] + two_x * b1 - b2;
        b2 = b1;
        b1 = bk;
    }
    return rows[0] + b1 * x - b2;
}

static long double minor_lu_ld(const long double* a, int n, uint64_t mask) {
    int idx[ORACLE_MAX_ORDER];
    long double m[ORACLE_MAX_ORDER * ORACLE_MAX_ORDER];
    int k = 0;
    for (int i = 0; i < n; ++i)
        if (mask & ((uint64_t)1 << i)) idx[k++] = i;
    for (int r = 0; r < k; ++r)
        for (int c = 0; c < k; ++c) m[r * k + c] = a[idx[r] * n + idx[c]];
    long double det = 1.0L;
    for (int col = 0; col < k; ++col) {
        int piv = col;
        for (int r = col + 1; r < k; ++r)
            if (fabsl(m[r * k + col]) > fabsl(m[piv * k + col])) piv = r;
        if (m[piv * k + col] == 0.0L) return 0.0L;
        if (piv != col) {
            for (int c = col; c < k; ++c) {
                const long double t = m[col * k + c];
                m[col * k + c] = m[piv * k + c];
                m[piv * k + c] = t;
            }
            det = -det;
        }
        const long double p = m[col * k + col];
        det *= p;
        for (int r = col + 1; r < k; ++r) {
            const long double f = m[r * k + col] / p;
            for (int c = col + 1; c < k; ++c) m[r * k + c] -= f * m[col * k + c];
        }
    }
    return det;
}

/* magnitude (may be NULL): the same prefactor times the connected recursion
 * run on absolute values, |dp|[m] = |a[m]| + sum |dp|[s] |a[m \ s]| (the
 * recursion's condition scale: the sum of the magnitudes of every term that
 * enters the top mask's value, through every level). */
static int integrand_one_set_ld(const oracle_scalars* s, const oracle_table* tu, const oracle_table* td,
                                const double* args, int order, int replica_count, long double* value,
                                long double* magnitude) {
    vertex vx[ORACLE_MAX_ORDER];
    long double mu[ORACLE_MAX_ORDER * ORACLE_MAX_ORDER], md[ORACLE_MAX_ORDER * ORACLE_MAX_ORDER];
    if (decode_vertices(s, args, order, replica_count, vx)) return ORACLE_BAD_INPUT;
    for (int idx = 0; idx < order * order; ++idx) {
        const int i = idx / order;
        const int j = idx - i * order;
        const int upper = (i != j) && (vx[i].tau_unit > vx[j].tau_unit);
        int corner;
        uint64_t index;
        double u, v;
        oracle_lookup_descriptor(vx[i].replica, vx[j].replica, vx[i].tau, vx[j].tau, vx[i].x, vx[i].y,
                                 vx[j].x, vx[j].y, s->beta, s->branch_eps, s->cheb_nu, s->cheb_nv, s->n1,
                                 s->n2, upper, &corner, &index, &u, &v);
        long double up, down;
        if (corner) {
            up = (long double)(upper ? tu->upper_corners[index] : tu->lower_corners[index]);
            down = (long double)(upper ? td->upper_corners[index] : td->lower_corners[index]);
        } else {
            up = chebyshev_2d_ld((upper ? tu->upper_coeffs : tu->lower_coeffs) + index, u, v, s->cheb_nu,
                                 s->cheb_nv);
            down = chebyshev_2d_ld((upper ? td->upper_coeffs : td->lower_coeffs) + index, u, v, s->cheb_nu,
                                   s->cheb_nv);
        }
        if (i == j) {
            up += (long double)s->diag_up_shift;
            down += (long double)s->diag_down_shift;
        }
        mu[idx] = up * (long double)s->scale;
        md[idx] = down * (long double)s->scale;
    }
    if (order < 2) return ORACLE_BAD_INPUT;  /* order 1 is the singleton form */
    const uint64_t count = (uint64_t)1 << order;
    long double* a = (long double*)malloc(count * sizeof(long double));
    long double* dp = (long double*)malloc(count * sizeof(long double));
    long double* adp = magnitude ? (long double*)malloc(count * sizeof(long double)) : NULL;
    if (!a || !dp || (magnitude && !adp)) {
        free(a);
        free(dp);
        free(adp);
        return ORACLE_BAD_INPUT;
    }
    a[0] = 0.0L;
    for (uint64_t m = 1; m < count; ++m) a[m] = minor_lu_ld(mu, order, m) * minor_lu_ld(md, order, m);
    dp[1] = a[1];
    if (adp) adp[1] = fabsl(a[1]);
    for (int bits = 2; bits <= order; ++bits) {
        for (uint64_t mask = 1; mask < count; mask += 2) {
            if (popcount64(mask) != bits) continue;
            long double acc = a[mask];
            long double mag = fabsl(a[mask]);
            for (uint64_t sub = (mask - 1) & mask; sub; sub = (sub - 1) & mask) {
                if (!(sub & 1u)) continue;
                acc -= dp[sub] * a[mask ^ sub];
                if (adp) mag += adp[sub] * fabsl(a[mask ^ sub]);
            }
            dp[mask] = acc;
            if (adp) adp[mask] = mag;
        }
    }
    long double pref = 1.0L;
    for (int i = 0; i < order; ++i) pref *= -(long double)replica_count;
    long double den = (long double)s->n1 * (long double)s->n2;
    for (int i = 2; i <= order; ++i) den *= (long double)i;
    *value = pref / den * dp[count - 1];
    if (magnitude) *magnitude = fabsl(pref / den) * adp[count - 1];
    free(a);
    free(dp);
    free(adp);
    return 0;
}

int oracle_integrand_ld(const oracle_scalars* s, const oracle_tables* t, const double* args, int order,
                        double* value) {
    return oracle_integrand_ld_parts(s, t, args, order, value, NULL);
}

int oracle_integrand_ld_parts(const oracle_scalars* s, const oracle_tables* t, const double* args, int order,
                              double* value, double* parts) {
    *value = 0.0;
    if (parts) parts[0] = parts[1] = parts[2] = parts[3] = 0.0;
    if (order <= 0 || order > ORACLE_MAX_ORDER) return ORACLE_BAD_INPUT;
    long double v[2], mag[2];
    const oracle_table* tabs[2][2] = {{&t->twisted_up, &t->twisted_down}, {&t->ordinary_up, &t->ordinary_down}};
    for (int set = 0; set < 2; ++set) {
        const int r = set == 0 ? 2 : 1;
        if (order == 1) {
            vertex vx[1];
            if (decode_vertices(s, args, 1, r, vx)) return ORACLE_BAD_INPUT;
            int corner;
            uint64_t index;
            double u, w;
            oracle_lookup_descriptor(vx[0].replica, vx[0].replica, vx[0].tau, vx[0].tau, vx[0].x, vx[0].y,
                                     vx[0].x, vx[0].y, s->beta, s->branch_eps, s->cheb_nu, s->cheb_nv, s->n1,
                                     s->n2, 0, &corner, &index, &u, &w);
            long double up, down;
            if (corner) {
                up = (long double)tabs[set][0]->lower_corners[index];
                down = (long double)tabs[set][1]->lower_corners[index];
            } else {
                up = chebyshev_2d_ld(tabs[set][0]->lower_coeffs + index, u, w, s->cheb_nu, s->cheb_nv);
                down = chebyshev_2d_ld(tabs[set][1]->lower_coeffs + index, u, w, s->cheb_nu, s->cheb_nv);
            }
            const long double su = up + (long double)s->diag_up_shift;
            const long double sd = down + (long double)s->diag_down_shift;
            const long double counter = (long double)s->diag_up_shift * (long double)s->diag_down_shift;
            v[set] = -(long double)r * (long double)s->u * (long double)s->beta * (su * sd - counter);
            mag[set] = (long double)r * fabsl((long double)s->u * (long double)s->beta) *
                       (fabsl(su * sd) + fabsl(counter));
        } else {
            const int st = integrand_one_set_ld(s, tabs[set][0], tabs[set][1], args, order, r, &v[set],
                                                parts ? &mag[set] : NULL);
            if (st) return st;
        }
    }
    *value = (double)(v[0] - 2.0L * v[1]);
    if (parts) {
        parts[0] = (double)v[0];
        parts[1] = (double)v[1];
        parts[2] = (double)mag[0];
        parts[3] = (double)mag[1];
    }
    return isfinite(*value) ? 0 : ORACLE_NONFINITE;
}

/* ---------------------------------------------------------- thread batch --- */

typedef struct batch_job {
    const oracle_scalars* s;
    const oracle_tables* t;
    const double* vertices;
    const int32_t* orders;
    int max_order;
    int all_subsets;  /* 1: all-subset values; 2: the long double truth */
    int64_t begin, end;
    double* values;
    int32_t* status;
    double* parts;    /* mode 2: the truth's twisted and ordinary parts, [batch][4] (parts and magnitudes), or NULL */
} batch_job;

static void* batch_worker(void* arg) {
    batch_job* job = (batch_job*)arg;
    for (int64_t c = job->begin; c < job->end; ++c) {
        const double* v = job->vertices + (size_t)c * (size_t)job->max_order * 4u;
        int st;
        if (job->all_subsets == 1) {
            st = oracle_all_subsets(job->s, job->t, v, job->max_order,
                                    job->values + (size_t)c * ((size_t)1 << job->max_order));
        } else if (job->all_subsets == 2) {
            st = oracle_integrand_ld_parts(job->s, job->t, v, job->orders[c], job->values + c,
                                           job->parts ? job->parts + 4 * c : NULL);
        } else {
            st = oracle_integrand(job->s, job->t, v, job->orders[c], job->values + c);
        }
        if (job->status) job->status[c] = st;
    }
    return NULL;
}

static int run_batch(batch_job proto, int64_t batch, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t tid[256];
    batch_job jobs[256];
    for (int w = 0; w < threads; ++w) {
        jobs[w] = proto;
        jobs[w].begin = batch * w / threads;
        jobs[w].end = batch * (w + 1) / threads;
        if (pthread_create(&tid[w], NULL, batch_worker, &jobs[w]) != 0) {
            for (int k = 0; k < w; ++k) pthread_join(tid[k], NULL);
            return -1;
        }
    }
    for (int w = 0; w < threads; ++w) pthread_join(tid[w], NULL);
    return 0;
}

int oracle_integrand_batch(const oracle_scalars* s, const oracle_tables* t,
                           const double* unit_vertices, const int32_t* orders, int64_t batch,
                           int max_order, double* values, int32_t* status, int threads) {
    batch_job proto = {s, t, unit_vertices, orders, max_order, 0, 0, 0, values, status, NULL};
    return run_batch(proto, batch, threads);
}

int oracle_all_subsets_batch(const oracle_scalars* s, const oracle_tables* t,
                             const double* unit_vertices, int envelope_order, int64_t batch,
                             double* values, int32_t* status, int threads) {
    batch_job proto = {s, t, unit_vertices, NULL, envelope_order, 1, 0, 0, values, status, NULL};
    return run_batch(proto, batch, threads);
}

int oracle_integrand_ld_batch(const oracle_scalars* s, const oracle_tables* t, const double* unit_vertices,
                              const int32_t* orders, int64_t batch, int max_order, double* values,
                              int32_t* status, int threads) {
    batch_job proto = {s, t, unit_vertices, orders, max_order, 2, 0, 0, values, status, NULL};
    return run_batch(proto, batch, threads);
}

int oracle_integrand_ld_parts_batch(const oracle_scalars* s, const oracle_tables* t, const double* unit_vertices,
                                    const int32_t* orders, int64_t batch, int max_order, double* values,
                                    double* parts, int32_t* status, int threads) {
    batch_job proto = {s, t, unit_vertices, orders, max_order, 2, 0, 0, values, status, parts};
    return run_batch(proto, batch, threads);
}

/* ------------------------------------------ order-1 diagonal observable --- */

/* chebyshev_uniform_integral_weight (diagonal_green_observable.h:57-67):
 * integral of T_k over [-1, 1]. */
static double uniform_integral_weight(int degree) {
    if (degree % 2 != 0) return 0.0;
    if (degree == 0) return 2.0;
    const double d = (double)degree;
    return 2.0 / (1.0 - d * d);
}

/* lower_diagonal_line_coefficients (:69-96): the lower-branch block of
 * (replica, replica, site, site) summed over v (T_b(1) = 1), per u row. */
static void diagonal_line(const oracle_table* t, int replica, int x, int y, int nu, int nv,
                          int n1, int n2, double* line) {
    const uint64_t base = sitepair_index(replica, replica, x, y, x, y, n1, n2) * (uint64_t)nu * (uint64_t)nv;
    const double* c = t->lower_coeffs + base;
    for (int a = 0; a < nu; ++a) {
        double sum = 0.0;
        for (int b = 0; b < nv; ++b) sum += c[(size_t)a * nv + b];
        line[a] = sum;
    }
}

/* integrate_chebyshev_line (:121-130) */
static double integrate_line(const double* line, int nu, double beta) {
    double integral = 0.0;
    for (int k = 0; k < nu; ++k) integral += line[k] * uniform_integral_weight(k);
    return beta * integral / 2.0;
}

/* integrate_chebyshev_line_product (:141-159) */
static double integrate_line_product(const double* lhs, const double* rhs, int nu, double beta) {
    double integral = 0.0;
    for (int i = 0; i < nu; ++i) {
        const double lv = lhs[i];
        for (int j = 0; j < nu; ++j) {
            const double rv = rhs[j];
            const int diff = i > j ? i - j : j - i;
            const double w = (uniform_integral_weight(i + j) + uniform_integral_weight(diff)) / 2.0;
            integral += lv * rv * w;
        }
    }
    return beta * integral / 2.0;
}

/* integrate_diagonal_shifted_product_from_tables (:161-180) */
static double diagonal_site_term(const oracle_table* up, const oracle_table* down, int replica, int x,
                                 int y, const oracle_scalars* s, double shift_up, double shift_down,
                                 double* up_line, double* down_line) {
    diagonal_line(up, replica, x, y, s->cheb_nu, s->cheb_nv, s->n1, s->n2, up_line);
    diagonal_line(down, replica, x, y, s->cheb_nu, s->cheb_nv, s->n1, s->n2, down_line);
    const double up_integral = integrate_line(up_line, s->cheb_nu, s->beta);
    const double down_integral = integrate_line(down_line, s->cheb_nu, s->beta);
    const double product = integrate_line_product(up_line, down_line, s->cheb_nu, s->beta);
    return product + shift_up * down_integral + shift_down * up_integral;
}

int oracle_diagonal_order1(const oracle_scalars* s, const oracle_tables* t, double alpha_up,
                           double alpha_down, double* out) {
    if (s->u == 0.0) return 1;
    const double shift_up = alpha_down / s->u;   /* diagonal_up_shift, :255-256 */
    const double shift_down = alpha_up / s->u;
    double* up_line = (double*)malloc(sizeof(double) * (size_t)s->cheb_nu);
    double* down_line = (double*)malloc(sizeof(double) * (size_t)s->cheb_nu);
    if (!up_line || !down_line) {
        free(up_line);
        free(down_line);
        return 2;
    }
    const double sites = (double)s->n1 * (double)s->n2;
    /* replica_log_partition_first_order_density_typed (:237-273) */
    double twisted_sum = 0.0;
    for (int replica = 0; replica < 2; ++replica)
        for (int y = 0; y < s->n2; ++y)
            for (int x = 0; x < s->n1; ++x)
                twisted_sum += diagonal_site_term(&t->twisted_up, &t->twisted_down, replica, x, y, s,
                                                  shift_up, shift_down, up_line, down_line);
    const double twisted = -s->u * twisted_sum / sites;
    /* ordinary_log_partition_first_order_density_typed (:275-303) */
    double ordinary_sum = 0.0;
    for (int y = 0; y < s->n2; ++y)
        for (int x = 0; x < s->n1; ++x)
            ordinary_sum += diagonal_site_term(&t->ordinary_up, &t->ordinary_down, 0, x, y, s, shift_up,
                                               shift_down, up_line, down_line);
    const double ordinary = -s->u * ordinary_sum / sites;
    free(up_line);
    free(down_line);
    /* normalized_log_partition_first_order_density_dd (:305-323) */
    out[0] = twisted - 2.0 * ordinary;
    out[1] = twisted;
    out[2] = ordinary;
    return 0;
}

/* ------------------------------------------------------- MCMCMC chain --- */

#define MT64_N 312
#define MT64_M 156

void oracle_mt64_seed(oracle_mt64* g, uint64_t seed) {
    g->mt[0] = seed;
    for (int i = 1; i < MT64_N; ++i) {
        const uint64_t x = g->mt[i - 1];
        g->mt[i] = 6364136223846793005ULL * (x ^ (x >> 62)) + (uint64_t)i;
    }
    g->index = MT64_N;
}

uint64_t oracle_mt64_next(oracle_mt64* g) {
    const uint64_t upper = 0xFFFFFFFF80000000ULL, lower = 0x7FFFFFFFULL, matrix = 0xB5026F5AA96619E9ULL;
    if (g->index >= MT64_N) {
        for (int i = 0; i < MT64_N; ++i) {
            const uint64_t x = (g->mt[i] & upper) | (g->mt[(i + 1) % MT64_N] & lower);
            g->mt[i] = g->mt[(i + MT64_M) % MT64_N] ^ (x >> 1) ^ ((x & 1ULL) ? matrix : 0ULL);
        }
        g->index = 0;
    }
    uint64_t y = g->mt[g->index++];
    y ^= (y >> 29) & 0x5555555555555555ULL;
    y ^= (y << 17) & 0x71D67FFFEDA60000ULL;
    y ^= (y << 37) & 0xFFF7EEE000000000ULL;
    y ^= y >> 43;
    return y;
}

double oracle_canonical(oracle_mt64* g) {
    const double r = (double)oracle_mt64_next(g) / 18446744073709551616.0;
    return r >= 1.0 ? nextafter(1.0, 0.0) : r;
}

int oracle_uniform_int(oracle_mt64* g, int n) {
    const uint64_t range = (uint64_t)n;
    unsigned __int128 product = (unsigned __int128)oracle_mt64_next(g) * range;
    uint64_t low = (uint64_t)product;
    if (low < range) {
        const uint64_t threshold = (0 - range) % range;
        while (low < threshold) {
            product = (unsigned __int128)oracle_mt64_next(g) * range;
            low = (uint64_t)product;
        }
    }
    return (int)(product >> 64);
}

/* binomial_as_double (mcmcmc_sampler.h:174-185): exact for the orders used. */
static double binomial_double(int n, int k) {
    if (k < 0 || k > n) return 0.0;
    if (k > n - k) k = n - k;
    uint64_t r = 1;
    for (int i = 1; i <= k; ++i) r = r * (uint64_t)(n - k + i) / (uint64_t)i;
    return (double)r;
}

/* adapt_mcmcmc_lambdas (mcmcmc_sampler.h:579-600) */
static void adapt_lambdas(double* lambdas, int order_min, int order_max, double rate, uint64_t* counts) {
    uint64_t total = 0;
    for (int o = order_min; o <= order_max; ++o) total += counts[o];
    if (total == 0) return;
    const int order_count = order_max - order_min + 1;
    const double target = 1.0 / (double)order_count;
    for (int o = order_min; o <= order_max; ++o) {
        const double actual = ((double)counts[o] + 1.0) / ((double)total + (double)order_count);
        lambdas[o] *= exp(rate * log(target / actual));
    }
}

/* FactorizedHistogramSeed (mcmcmc_seed.h:71-229); bins == 0: the uniform seed. */
typedef struct hist_seed {
    int bins, n1, n2, sites;
    const double *tau_prob, *space_prob, *rep_prob;
    double *tau_cdf, *space_cdf, *rep_cdf;
} hist_seed;

/* unit_coordinate_to_index (mcmcmc_seed.h:30-39) */
static int unit_index(double value, int extent) {
    const int index = (int)floor(value * (double)extent);
    if (index < 0) return 0;
    if (index >= extent) return extent - 1;
    return index;
}

/* build_cdfs (:190-203) */
static void build_cdf(const double* prob, int columns, int rows, double* cdf) {
    for (int r = 0; r < rows; ++r) {
        double cumulative = 0.0;
        for (int c = 0; c < columns; ++c) {
            cumulative += prob[r * columns + c];
            cdf[r * columns + c] = cumulative;
        }
        cdf[r * columns + columns - 1] = 1.0;
    }
}

/* sample_from_row (:205-218): std::lower_bound (binary search for the first
 * entry not below the draw) of a canonical draw; past the end: the last column */
static int sample_row(const double* cdf, int columns, int row, oracle_mt64* rng) {
    const double threshold = oracle_canonical(rng);
    const double* b = cdf + (size_t)row * columns;
    int first = 0, len = columns;
    while (len > 0) {
        const int half = len >> 1;
        if (b[first + half] < threshold) {
            first += half + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    return first == columns ? columns - 1 : first;
}

/* sample_child_from_parent (:106-128) */
static void hist_child(const hist_seed* h, const double* parent, oracle_mt64* rng, double* child) {
    const int child_tau = sample_row(h->tau_cdf, h->bins, unit_index(parent[0], h->bins), rng);
    const int parent_site = unit_index(parent[1], h->n1) * h->n2 + unit_index(parent[2], h->n2);
    const int child_site = sample_row(h->space_cdf, h->sites, parent_site, rng);
    const int child_x = child_site / h->n2;
    const int child_y = child_site - child_x * h->n2;
    const int child_rep = sample_row(h->rep_cdf, 2, unit_index(parent[3], 2), rng);
    child[0] = ((double)child_tau + oracle_canonical(rng)) / (double)h->bins;
    child[1] = ((double)child_x + oracle_canonical(rng)) / (double)h->n1;
    child[2] = ((double)child_y + oracle_canonical(rng)) / (double)h->n2;
    child[3] = ((double)child_rep + oracle_canonical(rng)) / 2.0;
}

/* density_child_given_parent (:130-150) */
static double hist_density(const hist_seed* h, const double* child, const double* parent) {
    const double tau_d = h->tau_prob[unit_index(parent[0], h->bins) * h->bins + unit_index(child[0], h->bins)] *
                         (double)h->bins;
    const int ps = unit_index(parent[1], h->n1) * h->n2 + unit_index(parent[2], h->n2);
    const int cs = unit_index(child[1], h->n1) * h->n2 + unit_index(child[2], h->n2);
    const double space_d = h->space_prob[ps * h->sites + cs] * (double)h->sites;
    const double rep_d = h->rep_prob[unit_index(parent[3], 2) * 2 + unit_index(child[3], 2)] * 2.0;
    return tau_d * space_d * rep_d;
}

/* compute_conditional_generation_probabilities_typed_into<double>
 * (mcmcmc_sampler.h:252-335); cd is [2^n][n] scratch. Returns 4 on a
 * negative or non-finite seed density. */
static int conditional_probabilities(const hist_seed* h, const double* v, int n, double* prob, double* cd) {
    double sd[64 * 64];
    for (int c = 0; c < n; ++c)
        for (int p = 0; p < n; ++p) {
            if (c == p) {
                sd[c * n + p] = 0.0;
                continue;
            }
            const double d = hist_density(h, v + 4 * c, v + 4 * p);
            if (d < 0.0 || !isfinite(d)) return 4;
            sd[c * n + p] = d;
        }
    const uint64_t count = (uint64_t)1 << n, full = count - 1;
    for (int c = 0; c < n; ++c) {
        double sum = 0.0;
        for (int p = 0; p < n; ++p) sum += sd[c * n + p];
        cd[c] = sum;
    }
    for (uint64_t m = 0; m < count; ++m) prob[m] = 0.0;
    prob[0] = 1.0;
    for (uint64_t gm = 1; gm < full; ++gm) {
        const uint64_t low = gm & (~gm + 1);
        const int removed = __builtin_ctzll(low);
        const uint64_t prev = gm ^ low;
        for (int c = 0; c < n; ++c) {
            double d = cd[prev * n + c] - sd[c * n + removed];
            if (d < 0.0 && d > -1.0e-12) d = 0.0;
            cd[gm * n + c] = d;
        }
        const int gc = __builtin_popcountll(gm), pc = n - gc;
        double sum = 0.0;
        for (int c = 0; c < n; ++c) {
            const uint64_t cb = (uint64_t)1 << c;
            if (!(gm & cb)) continue;
            sum += prob[gm ^ cb] * cd[gm * n + c];
        }
        prob[gm] = sum / ((double)gc * (double)pc);
    }
    prob[full] = 0.0;
    return 0;
}

/* run_mcmcmc_step (mcmcmc_sampler.h:524-577) with the uniform seed kernel, or
 * the histogram seed when h->bins > 0. */
static int mcmcmc_step(const oracle_scalars* s, const oracle_tables* t, int order_min, int order_max, int envelope,
                       const double* lambdas, const double* inv_binom, double* vertices, oracle_mt64* rng,
                       double* values, double* fluxes, double* weights, uint64_t* chosen_out, double* norm_out,
                       double* signal, const hist_seed* h, double* cprob, double* cd) {
    if (oracle_all_subsets(s, t, vertices, envelope, values) & ORACLE_NONFINITE) return 1;
    const uint64_t full_mask = ((uint64_t)1 << envelope) - 1;
    if (h->bins > 0) {
        const int rc = conditional_probabilities(h, vertices, envelope, cprob, cd);
        if (rc) return rc;
    }
    const uint64_t subsets = (uint64_t)1 << envelope;
    double norm = 0.0;
    int idx = 0;
    for (uint64_t mask = 1; mask < subsets; ++mask) {
        const int o = __builtin_popcountll(mask);
        if (o < order_min || o > order_max) continue;
        const double flux = lambdas[o] * values[mask] * (h->bins > 0 ? cprob[full_mask ^ mask] : 1.0);
        const double w = fabs(flux) * inv_binom[o];
        fluxes[idx] = flux;
        weights[idx] = w;
        norm += w;
        ++idx;
    }
    /* sample_weighted_candidate_mask (:225-250) */
    if (!(norm > 0.0) || !isfinite(norm)) return 2;
    const double threshold = oracle_canonical(rng) * (norm - 0.0) + 0.0;
    double cumulative = 0.0;
    uint64_t chosen = 0, last_positive = 0;
    int found = 0;
    idx = 0;
    for (uint64_t mask = 1; mask < subsets && !found; ++mask) {
        const int o = __builtin_popcountll(mask);
        if (o < order_min || o > order_max) continue;
        const double w = weights[idx++];
        if (!(w > 0.0)) continue;
        if (isfinite(w)) last_positive = mask;
        cumulative += w;
        if (cumulative > threshold) {
            chosen = mask;
            found = 1;
        }
    }
    if (!found) chosen = last_positive;
    for (int o = 0; o <= envelope; ++o) signal[o] = 0.0;
    idx = 0;
    for (uint64_t mask = 1; mask < subsets; ++mask) {
        const int o = __builtin_popcountll(mask);
        if (o < order_min || o > order_max) continue;
        const double time = fluxes[idx++] / norm;
        signal[o] += time * inv_binom[o];
    }
    /* create_next_vertices_from_seed_into (:380-400), uniform seed (mcmcmc_seed.h:51-55) */
    double next[64 * 4];
    int size = 0;
    for (int i = 0; i < envelope; ++i)
        if (chosen & ((uint64_t)1 << i)) {
            for (int k = 0; k < 4; ++k) next[4 * size + k] = vertices[4 * i + k];
            ++size;
        }
    while (size < envelope) {
        const int parent = oracle_uniform_int(rng, size);
        if (h->bins > 0) {
            hist_child(h, next + 4 * parent, rng, next + 4 * size);
        } else {
            for (int k = 0; k < 4; ++k) next[4 * size + k] = oracle_canonical(rng); /* uniform: parent ignored */
        }
        ++size;
    }
    memcpy(vertices, next, sizeof(double) * 4 * (size_t)envelope);
    *chosen_out = chosen;
    *norm_out = norm;
    return 0;
}

static int mcmcmc_chain(const oracle_scalars* s, const oracle_tables* t, int order_min, int order_max, int envelope,
                        const double* lambdas_in, int warmup, int adapt_interval, double adapt_rate, int production,
                        uint64_t seed, const hist_seed* h, uint64_t* chosen, double* norms, double* signal,
                        double* vertices_out, double* lambdas_out, uint64_t* rng_out) {
    oracle_mt64 rng;
    oracle_mt64_seed(&rng, seed);
    double vertices[64 * 4];
    for (int i = 0; i < envelope * 4; ++i) vertices[i] = oracle_canonical(&rng); /* sample_uniform_vertex_set */
    double lambdas[65], inv_binom[65];
    uint64_t counts[65];
    for (int o = 0; o <= envelope; ++o) {
        lambdas[o] = lambdas_in[o];
        counts[o] = 0;
        inv_binom[o] = (o >= order_min && o <= order_max) ? 1.0 / binomial_double(envelope, o) : 0.0;
    }
    const size_t subsets = (size_t)1 << envelope;
    double* values = (double*)malloc(sizeof(double) * subsets);
    double* fluxes = (double*)malloc(sizeof(double) * subsets);
    double* weights = (double*)malloc(sizeof(double) * subsets);
    double* cprob = (double*)malloc(sizeof(double) * subsets);
    double* cd = (double*)malloc(sizeof(double) * subsets * (size_t)envelope);
    double step_signal[65];
    int rc = (values && fluxes && weights && cprob && cd) ? 0 : 3;
    int k = 0;
    for (int step = 0; rc == 0 && step < warmup; ++step, ++k) {
        rc = mcmcmc_step(s, t, order_min, order_max, envelope, lambdas, inv_binom, vertices, &rng, values, fluxes,
                         weights, &chosen[k], &norms[k], step_signal, h, cprob, cd);
        if (rc) break;
        ++counts[__builtin_popcountll(chosen[k])];
        if ((step + 1) % adapt_interval == 0) {
            adapt_lambdas(lambdas, order_min, order_max, adapt_rate, counts);
            for (int o = 0; o <= envelope; ++o) counts[o] = 0;
        }
    }
    if (rc == 0 && warmup % adapt_interval != 0) {
        int pending = 0;
        for (int o = 0; o <= envelope; ++o) pending |= counts[o] != 0;
        if (pending) adapt_lambdas(lambdas, order_min, order_max, adapt_rate, counts);
    }
    for (int step = 0; rc == 0 && step < production; ++step, ++k) {
        rc = mcmcmc_step(s, t, order_min, order_max, envelope, lambdas, inv_binom, vertices, &rng, values, fluxes,
                         weights, &chosen[k], &norms[k], signal + (size_t)step * (envelope + 1), h, cprob, cd);
    }
    free(values);
    free(fluxes);
    free(weights);
    free(cprob);
    free(cd);
    if (rc) return rc;
    memcpy(vertices_out, vertices, sizeof(double) * 4 * (size_t)envelope);
    for (int o = 0; o <= envelope; ++o) lambdas_out[o] = lambdas[o];
    for (int i = 0; i < 8; ++i) rng_out[i] = oracle_mt64_next(&rng);
    return 0;
}

int oracle_mcmcmc_chain(const oracle_scalars* s, const oracle_tables* t, int order_min, int order_max,
                        int envelope, const double* lambdas_in, int warmup, int adapt_interval, double adapt_rate,
                        int production, uint64_t seed, uint64_t* chosen, double* norms, double* signal,
                        double* vertices_out, double* lambdas_out, uint64_t* rng_out) {
    const hist_seed none = {0, 0, 0, 0, NULL, NULL, NULL, NULL, NULL, NULL};
    return mcmcmc_chain(s, t, order_min, order_max, envelope, lambdas_in, warmup, adapt_interval, adapt_rate,
                        production, seed, &none, chosen, norms, signal, vertices_out, lambdas_out, rng_out);
}

int oracle_mcmcmc_chain_hist(const oracle_scalars* s, const oracle_tables* t, int order_min, int order_max,
                             int envelope, const double* lambdas_in, int warmup, int adapt_interval, double adapt_rate,
                             int production, uint64_t seed, int tau_bins, const double* tau_prob,
                             const double* space_prob, const double* replica_prob, uint64_t* chosen, double* norms,
                             double* signal, double* vertices_out, double* lambdas_out, uint64_t* rng_out) {
    hist_seed h;
    h.bins = tau_bins;
    h.n1 = s->n1;
    h.n2 = s->n2;
    h.sites = s->n1 * s->n2;
    h.tau_prob = tau_prob;
    h.space_prob = space_prob;
    h.rep_prob = replica_prob;
    h.tau_cdf = (double*)malloc(sizeof(double) * (size_t)tau_bins * tau_bins);
    h.space_cdf = (double*)malloc(sizeof(double) * (size_t)h.sites * h.sites);
    h.rep_cdf = (double*)malloc(sizeof(double) * 4);
    int rc = 3;
    if (h.tau_cdf && h.space_cdf && h.rep_cdf) {
        build_cdf(tau_prob, tau_bins, tau_bins, h.tau_cdf);
        build_cdf(space_prob, h.sites, h.sites, h.space_cdf);
        build_cdf(replica_prob, 2, 2, h.rep_cdf);
        rc = mcmcmc_chain(s, t, order_min, order_max, envelope, lambdas_in, warmup, adapt_interval, adapt_rate,
                          production, seed, &h, chosen, norms, signal, vertices_out, lambdas_out, rng_out);
    }
    free(h.tau_cdf);
    free(h.space_cdf);
    free(h.rep_cdf);
    return rc;
}

/* splitmix64_mcmcmc / derive_mcmcmc_seed (mcmcmc_sampler.h:159-172) */
static uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30U)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27U)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31U);
}

static uint64_t derive_seed(uint64_t base, uint64_t tag, uint64_t index) {
    uint64_t mixed = splitmix64(base ^ tag);
    mixed ^= 0x9e3779b97f4a7c15ULL * (index + 1ULL);
    return splitmix64(mixed);
}

/* FactorizedHistogramSeedAccumulator::normalize_rows (mcmcmc_seed.h:288-327) */
static void normalize_rows(const long double* counts, int columns, int rows, double mix_d, double pseudo_d,
                           double* out) {
    const long double uniform = 1.0L / (long double)columns;
    const long double mix = (long double)mix_d, pseudo = (long double)pseudo_d;
    for (int r = 0; r < rows; ++r) {
        long double row_sum = 0.0L;
        for (int c = 0; c < columns; ++c) row_sum += counts[r * columns + c];
        const long double denominator = row_sum + pseudo * (long double)columns;
        for (int c = 0; c < columns; ++c) {
            long double learned = uniform;
            if (denominator > 0.0L) learned = (counts[r * columns + c] + pseudo) / denominator;
            const long double probability = (1.0L - mix) * learned + mix * uniform;
            out[r * columns + c] = (double)probability;
        }
        double row_total = 0.0;
        for (int c = 0; c < columns; ++c) row_total += out[r * columns + c];
        if (row_total > 0.0 && isfinite(row_total))
            for (int c = 0; c < columns; ++c) out[r * columns + c] /= row_total;
    }
}

int oracle_learn_histogram(const oracle_scalars* s, const oracle_tables* t, int order_min, int order_max,
                           int envelope, int learning_steps, int tau_bins, double uniform_mix, double pseudo_count,
                           uint64_t base_seed, double* tau_out, double* space_out, double* replica_out,
                           double* total_weight_out) {
    const int sites = s->n1 * s->n2;
    long double* tau_c = (long double*)calloc((size_t)tau_bins * tau_bins, sizeof(long double));
    long double* space_c = (long double*)calloc((size_t)sites * sites, sizeof(long double));
    long double rep_c[4] = {0.0L, 0.0L, 0.0L, 0.0L};
    long double total = 0.0L;
    const size_t subsets = (size_t)1 << envelope;
    double* values = (double*)malloc(sizeof(double) * subsets);
    if (!tau_c || !space_c || !values) {
        free(tau_c);
        free(space_c);
        free(values);
        return 3;
    }
    oracle_mt64 rng;
    oracle_mt64_seed(&rng, derive_seed(base_seed, 0x484953544F534545ULL, 0));
    double v[64 * 4];
    for (int step = 0; step < learning_steps; ++step) {
        for (int i = 0; i < envelope * 4; ++i) v[i] = oracle_canonical(&rng); /* sample_uniform_vertex_set */
        if (oracle_all_subsets(s, t, v, envelope, values) & ORACLE_NONFINITE) {
            free(tau_c);
            free(space_c);
            free(values);
            return 1; /* the all-subset evaluation throws on a non-finite value */
        }
        for (uint64_t mask = 1; mask < subsets; ++mask) {
            const int order = __builtin_popcountll(mask);
            if (order < order_min || order > order_max || order < 2) continue;
            const double value = values[mask];
            if (!isfinite(value)) continue;
            const long double subset_weight = (long double)fabs(value) / (long double)binomial_double(envelope, order);
            const long double pair_weight = subset_weight / (long double)(order * (order - 1));
            if (!(pair_weight > 0.0L)) continue;
            for (int p = 0; p < envelope; ++p) {
                if (!(mask & ((uint64_t)1 << p))) continue;
                for (int c = 0; c < envelope; ++c) {
                    if (c == p || !(mask & ((uint64_t)1 << c))) continue;
                    /* add_pair (mcmcmc_seed.h:249-258) */
                    if (!(pair_weight > 0.0L) || !isfinite((double)pair_weight)) continue;
                    const double* pv = v + 4 * p;
                    const double* cv = v + 4 * c;
                    tau_c[unit_index(pv[0], tau_bins) * tau_bins + unit_index(cv[0], tau_bins)] += pair_weight;
                    const int ps = unit_index(pv[1], s->n1) * s->n2 + unit_index(pv[2], s->n2);
                    const int cs = unit_index(cv[1], s->n1) * s->n2 + unit_index(cv[2], s->n2);
                    space_c[ps * sites + cs] += pair_weight;
                    rep_c[unit_index(pv[3], 2) * 2 + unit_index(cv[3], 2)] += pair_weight;
                    total += pair_weight;
                }
            }
        }
    }
    normalize_rows(tau_c, tau_bins, tau_bins, uniform_mix, pseudo_count, tau_out);
    normalize_rows(space_c, sites, sites, uniform_mix, pseudo_count, space_out);
    normalize_rows(rep_c, 2, 2, uniform_mix, pseudo_count, replica_out);
    *total_weight_out = (double)total;
    free(tau_c);
    free(space_c);
    free(values);
    return 0;
}
