// Host check of the compact minors workspace (compact_minors_layout and the
// list placement in cdet_kernels.cuh), for every batch order nmax <= 10 and
// matrix order n <= nmax, with one and two spins, with and without A:
//  - every level list lies inside its arena;
//  - list L_k never covers a shifted minor that is written while L_k is still
//    read (the minors below 2^(k+1), and for L_{n-2}, which the last level reads
//    while it writes its minors, all of [0, 2^n));
//  - the two lists of a level (L_k read, L_{k+1} written) never meet;
//  - the arena keeps 2^nmax elements after the minors for the recursion arrays
//    of the forms that run the CDet on the same warp.
// Prints each violation and exits non-zero if there is one.
#include "cdet_kernels.cuh"

#include <cstdio>

using namespace cdet;

static int failures = 0;

#define CHECK(cond, ...)                 \
    do {                                 \
        if (!(cond)) {                   \
            ++failures;                  \
            std::printf(__VA_ARGS__);    \
            std::printf("\n");           \
        }                                \
    } while (0)

static bool disjoint(long a0, long a1, long b0, long b1) { return a1 <= b0 || b1 <= a0; }

int main() {
    int layouts = 0;
    for (int nmax = 1; nmax <= kCompactMaxOrder; ++nmax) {
        for (int two = 0; two < 2; ++two) {
            for (int with_a = 0; with_a < 2; ++with_a) {
                const WsLayout l = compact_minors_layout(nmax, two != 0, with_a != 0);
                const long arena = l.arena;
                ++layouts;
                CHECK(arena >= (2L << nmax), "nmax %d: arena %ld below 2^(nmax+1)", nmax, arena);
                CHECK(static_cast<long>(l.shifted_down) == static_cast<long>(l.shifted_up) + arena,
                      "nmax %d: spin-down arena does not follow the spin-up one", nmax);
                CHECK(static_cast<long>(l.total) == static_cast<long>(l.shifted_up) + arena * (two ? 2 : 1),
                      "nmax %d: total %zu", nmax, l.total);
                CHECK(!with_a || static_cast<long>(l.shifted_up) >= static_cast<long>(nmax) * nmax,
                      "nmax %d: A overlaps the spin-up arena", nmax);
                CHECK(static_cast<long>(l.old_list) >= static_cast<long>(l.shifted_up) + (1L << nmax),
                      "nmax %d: recursion arrays overlap the spin-up minors", nmax);
                CHECK(static_cast<long>(l.new_list) + (1L << (nmax - 1)) <= static_cast<long>(l.shifted_up) + arena,
                      "nmax %d: recursion arrays leave the spin-up arena", nmax);
                for (int n = 1; n <= nmax; ++n) {
                    const int last = n >= 2 ? n - 2 : 0;  // L_0 .. L_{n-2} (L_0 alone at n = 1)
                    for (int k = 0; k <= last; ++k) {
                        const long o = compact_list_offset(n, k, static_cast<int>(arena));
                        const long e = o + compact_list_doubles(n, k);
                        CHECK(o >= 0 && e <= arena, "nmax %d n %d: L_%d [%ld, %ld) outside the arena %ld", nmax, n,
                              k, o, e, arena);
                        const long live = (n >= 2 && k == n - 2) ? (1L << n) : (2L << k);
                        CHECK(o >= live, "nmax %d n %d: L_%d at %ld covers minors written below %ld", nmax, n, k, o,
                              live);
                        if (k + 1 <= last) {
                            const long o2 = compact_list_offset(n, k + 1, static_cast<int>(arena));
                            const long e2 = o2 + compact_list_doubles(n, k + 1);
                            CHECK(disjoint(o, e, o2, e2), "nmax %d n %d: L_%d [%ld, %ld) meets L_%d [%ld, %ld)", nmax,
                                  n, k, o, e, k + 1, o2, e2);
                        }
                    }
                }
            }
        }
    }
    std::printf("%d layouts checked, %d violations\n", layouts, failures);
    return failures == 0 ? 0 : 1;
}
