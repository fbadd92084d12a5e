// Drop-in replacement of the reference's size-bound driver,
// circlecover::rectangle_size_bound::find_critical_intervals()
// (reference: rectangle_size_bound/rectangle_size_bound.cu:312-382, called
// from prover.cpp:35), on top of the C ABI in include/circlecover_gb300.h.
//
// Same root box (lambda in [1, 2.5], every squared radius in [0, 9/64];
// values.hpp:28-35), same split counts (rectangle_size_bound.cu:36-62), same
// stdout (banner, one "Critical: " line per critical box in the reference's
// final order, Variables' text format with 19-digit intervals), same Ctrl-C
// behaviour (the refinement stops and the previous generation's result is
// printed).  The environment variable CC_SB_LAMBDA_MAX narrows the lambda
// range for short runs, and CC_SB_GRID="la:r1,...,r6:la_gen:s1,...,s6:gens"
// replaces the split counts.  Leaves that reached a trap site (where the
// reference would have aborted the run) are printed with a "Trapped: "
// prefix instead.
#include <vector>

#include "dropin.hpp"

namespace circlecover {
namespace rectangle_size_bound {
void find_critical_intervals();
}

namespace dropin {

// reference: rectangle_size_bound/variables.hpp:112-118
std::ostream& operator<<(std::ostream& o, const cc_sb_box& b) {
    o << "λ = " << b.la;
    for (int i = 0; i < 6; ++i) o << ", r²_" << (i + 1) << " = " << b.r[i];
    return o;
}

cc_sb_grid reference_sb_grid() {
    cc_sb_grid g{};
    const int init[6] = {128, 128, 64, 64, 64, 64};
    const int subdiv[6] = {32, 32, 16, 16, 16, 32};
    g.la_splits_init = 256;
    g.la_splits_gen = 64;
    for (int k = 0; k < 6; ++k) {
        g.r_splits_init[k] = init[k];
        g.r_splits_gen[k] = subdiv[k];
    }
    g.num_generations = 1;
    if (const char* e = std::getenv("CC_SB_GRID")) {
        const std::vector<std::string> f = split_fields(e);
        if (f.size() != 5) throw std::runtime_error("CC_SB_GRID: la:r1,...,r6:la_gen:s1,...,s6:gens");
        parse_ints(f[0], &g.la_splits_init, 1);
        parse_ints(f[1], g.r_splits_init, 6);
        parse_ints(f[2], &g.la_splits_gen, 1);
        parse_ints(f[3], g.r_splits_gen, 6);
        parse_ints(f[4], &g.num_generations, 1);
    }
    return g;
}

}  // namespace dropin
}  // namespace circlecover

void circlecover::rectangle_size_bound::find_critical_intervals() {
    using namespace circlecover::dropin;
    begin_case("Critical intervals for rectangles with small disks");
    std::cerr << "Size bound: r <= " << 0.375 << ", critical ratio: " << 0.61 << std::endl;
    cc_handle* h = nullptr;
    check(nullptr, cc_create(&h, 0), "cc_create");
    const double w = 9.0 / 64.0;
    double la_hi = 2.5;
    if (const char* e = std::getenv("CC_SB_LAMBDA_MAX")) la_hi = std::strtod(e, nullptr);
    cc_sb_box root{{1.0, la_hi}, {{0.0, w}, {0.0, w}, {0.0, w}, {0.0, w}, {0.0, w}, {0.0, w}}};
    cc_sb_grid grid = reference_sb_grid();

    std::cerr << "Initializing; press Ctrl-C during the refinement to use the best result achieved so far..."
              << std::endl;
    g_interrupts.store(0);
    g_active.store(h);
    void (*previous)(int) = std::signal(SIGINT, on_sigint);
    cc_sb_box* crit = nullptr;
    uint32_t* flags = nullptr;
    size_t n = 0;
    cc_sb_prove_stats stats;
    int st = cc_sb_prove(h, &root, &grid, &crit, &n, &flags, &stats);
    std::signal(SIGINT, previous);
    g_active.store(nullptr);
    check(h, st, "cc_sb_prove");
    std::cerr << "Generations run: " << stats.generations_run << ", criticals: " << n << ", leaves: " << stats.leaf_evals
              << ", " << stats.seconds << " s" << std::endl;
    for (size_t i = 0; i < n; ++i) std::cout << (flags[i] ? "Trapped: " : "Critical: ") << crit[i] << std::endl;
    cc_free(crit);
    cc_free(flags);
    cc_destroy(h);
    end_case();
}
