// cdet_gb300.hpp - C++20 drop-in adapter over the C ABI in cdet_gb300.h.
//
// Gives the reference's MCMCMC driver the two integrand entry points it calls,
// with the reference's signatures, argument meaning and exceptions:
//
//   double evaluate_cdet_density_integrand_double(const std::vector<UnitVertex>&)
//       (include/cdet/cdet_integrand_evaluator.h:542-560)
//   void evaluate_cdet_density_all_subset_integrands_double_into(
//       const std::vector<UnitVertex>&, std::vector<double>&)        (:562-583)
//   std::vector<double> evaluate_cdet_density_all_subset_integrands_double(...)  (:585-590)
//
// The reference reads its parameters and tables from process globals
// (parameters.h:11-91); here one Integrand object holds them on the GPU and
// install() makes it the one the free functions use. A driver that evaluates
// many proposals per step calls Integrand::evaluate_batch instead.
#pragma once

#include "cdet_gb300.h"

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace cdet_gb300 {

// UnitVertex (cdet_integrand_evaluator.h:16-21): coordinates in [0, 1).
struct UnitVertex {
    double tau = 0.0;
    double x = 0.0;
    double y = 0.0;
    double replica = 0.0;
};

// One PiecewiseChebyshevTable<double> (replica_chebyshev_tables.h:25-33).
struct TableView {
    const std::vector<double>* upper_coeffs = nullptr;
    const std::vector<double>* lower_coeffs = nullptr;
    const std::vector<double>* upper_corners = nullptr;
    const std::vector<double>* lower_corners = nullptr;
};

inline void check(int rc) {
    if (rc != CDET_OK) throw std::runtime_error(cdet_last_error());
}

class Integrand {
public:
    Integrand(const cdet_runtime_scalars& scalars, int device = 0) {
        cdet_context* ctx = nullptr;
        check(cdet_create(&scalars, device, &ctx));
        ctx_.reset(ctx);
    }

    // Copies one of the four tables (kind = cdet_table_kind) to the GPU.
    void upload(int kind, const TableView& t) {
        const cdet_table_view view{t.upper_coeffs->data(), t.lower_coeffs->data(),
                                   t.upper_corners->data(), t.lower_corners->data()};
        check(cdet_upload_table(ctx_.get(), kind, &view, t.upper_coeffs->size(),
                                t.upper_corners->size()));
    }

    // The reference's ALPHA_UP == ALPHA_DOWN sharing (load_data.h:70-91).
    void alias(int kind, int source_kind) { check(cdet_alias_table(ctx_.get(), kind, source_kind)); }

    void set_assembly(int mode) { check(cdet_set_assembly(ctx_.get(), mode)); }

    double integrand(const std::vector<UnitVertex>& vertices) {
        const int order = static_cast<int>(vertices.size());
        if (order <= 0) throw std::runtime_error("The replica integrand is defined only for order >= 1");
        double value = 0.0;
        int32_t status = 0;
        const int32_t orders = order;
        const int rc = cdet_integrand_host(ctx_.get(), &vertices[0].tau, &orders, 1, order, &value, &status);
        if (status & CDET_CONFIG_NONFINITE) throw std::runtime_error("Error (integrand): Value is not finite");
        if (status & CDET_CONFIG_BAD_INPUT) throw std::runtime_error("Error (integrand): vertex coordinates rejected");
        check(rc);
        return value;
    }

    void all_subsets_into(const std::vector<UnitVertex>& vertices, std::vector<double>& values) {
        const int envelope = static_cast<int>(vertices.size());
        if (envelope <= 1)
            throw std::runtime_error("The all-subset replica integrand is defined only for envelope order >= 2");
        values.resize(std::size_t{1} << envelope);
        int32_t status = 0;
        const int rc = cdet_all_subsets_host(ctx_.get(), &vertices[0].tau, envelope, 1, values.data(), &status);
        if (status & CDET_CONFIG_NONFINITE)
            throw std::runtime_error("Error (all-subset integrand): Value is not finite");
        if (status & CDET_CONFIG_BAD_INPUT)
            throw std::runtime_error("Error (all-subset integrand): vertex coordinates rejected");
        check(rc);
    }

    // Many configurations at once: vertices [batch][max_order], orders [batch].
    void evaluate_batch(const std::vector<UnitVertex>& vertices, const std::vector<int32_t>& orders,
                        int max_order, std::vector<double>& values, std::vector<int32_t>& status) {
        const int64_t batch = static_cast<int64_t>(orders.size());
        values.resize(orders.size());
        status.resize(orders.size());
        const int rc = cdet_integrand_host(ctx_.get(), &vertices[0].tau, orders.data(), batch, max_order,
                                           values.data(), status.data());
        if (rc != CDET_OK && rc != CDET_ERR_VALUE) check(rc);
    }

    // Deterministic order-1 diagonal observable of the uploaded tables
    // (diagonal_observable_density_dd, diagonal_green_observable.h:357-366):
    // the normalised coefficient twisted - 2 ordinary. The reference reads
    // ALPHA_UP and ALPHA_DOWN from its globals; pass their double values.
    double diagonal_observable_density(double alpha_up, double alpha_down) {
        double out[3] = {0.0, 0.0, 0.0};
        check(cdet_diagonal_order1_density(ctx_.get(), alpha_up, alpha_down, out));
        return out[0];
    }

    // Makes this object the one the free functions below use.
    void install() { current() = this; }

    static Integrand*& current() {
        static Integrand* instance = nullptr;
        return instance;
    }

private:
    struct Deleter {
        void operator()(cdet_context* c) const { cdet_destroy(c); }
    };
    std::unique_ptr<cdet_context, Deleter> ctx_;
};

static_assert(sizeof(UnitVertex) == 4 * sizeof(double), "UnitVertex is passed as [order][4] doubles");

inline Integrand& installed() {
    Integrand* p = Integrand::current();
    if (!p) throw std::runtime_error("Green-function tables have not been uploaded (no Integrand installed)");
    return *p;
}

inline double evaluate_cdet_density_integrand_double(const std::vector<UnitVertex>& vertices) {
    return installed().integrand(vertices);
}

inline void evaluate_cdet_density_all_subset_integrands_double_into(const std::vector<UnitVertex>& vertices,
                                                                    std::vector<double>& values) {
    installed().all_subsets_into(vertices, values);
}

inline std::vector<double> evaluate_cdet_density_all_subset_integrands_double(
    const std::vector<UnitVertex>& vertices) {
    std::vector<double> values;
    evaluate_cdet_density_all_subset_integrands_double_into(vertices, values);
    return values;
}

}  // namespace cdet_gb300
