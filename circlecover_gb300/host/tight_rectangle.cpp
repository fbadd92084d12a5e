// Drop-in replacement of the reference's tight-rectangle driver,
// circlecover::tight_rectangle::find_critical_intervals()
// (reference: tight_rectangle/tight_rectangle.cu:458-537, called from
// prover.cpp:34), on top of the C ABI in include/circlecover_gb300.h.
//
// Same split counts, same stdout (banner, the two- and three-disk summaries
// with 19-digit intervals), same Ctrl-C behaviour: the first SIGINT stops the
// refinement after the current generation and the result so far is used,
// the second one exits (reference: interrupt.cpp:30-46).  With
// CC_TIGHT_CHECKPOINT=<file> the state is saved after every generation and
// a later run resumes from it.  Errors that the
// reference reports by throwing std::system_error/std::logic_error are thrown
// here as std::runtime_error with the library's message.
#include <cstdio>

#include "dropin.hpp"

namespace circlecover {
namespace tight_rectangle {
void find_critical_intervals();
}

namespace dropin {

// reference: tight_rectangle.cu:539-545
std::ostream& operator<<(std::ostream& o, const cc_tight_box& b) {
    o << "λ = " << b.la;
    for (int i = 0; i < 4; ++i) o << ", r²_" << (i + 1) << " = " << b.r[i];
    return o;
}

void print_summary(const cc_tight_summary_t& r) {
    if (r.have_range_2d) {
        std::cout << "Two disks: Range for lambda that contains 2-disk critical intervals: " << r.la_range_2d
                  << "; maximal distances from theoretical values: " << std::endl;
        std::cout << "\tr_1^2: " << r.dist_r1_2d << ", r_2^2: " << r.dist_r2_2d << ", R_3 <= " << r.ub_R3_2d
                  << ", h_1 >= " << r.lb_h1_2d << ", lambda / S_1 <= " << r.ub_la_by_S1 << std::endl;
        std::cout << "\tDominating criticals for r_1: " << std::endl;
        std::cout << "\t\t" << r.dist_r1_2d_criticals[0] << std::endl;
        std::cout << "\t\t" << r.dist_r1_2d_criticals[1] << std::endl;
        std::cout << "\tDominating criticals for r_2: " << std::endl;
        std::cout << "\t\t" << r.dist_r2_2d_criticals[0] << std::endl;
        std::cout << "\t\t" << r.dist_r2_2d_criticals[1] << std::endl;
    }
    if (r.have_range_3d) {
        std::cout << "Three disks: Range for lambda that contains 3-disk critical intervals: " << r.la_range_3d
                  << "; maximal distances from theoretical values: " << std::endl;
        std::cout << "\tr_1^2: " << r.dist_r1_3d << ", r_2^2: " << r.dist_r2_3d << ", r_3^2: " << r.dist_r3_3d
                  << ", R_4 <= " << r.ub_R4_3d << std::endl;
        std::cout << "\tS_1: " << r.S1 << ", h_2: " << r.h2 << ", S_3: " << r.S3 << ", pocket width <= " << r.pocket_width_3d
                  << std::endl;
        std::cout << "\tDominating criticals for r_1: " << std::endl;
        std::cout << "\t\t" << r.dist_r1_3d_criticals[0] << std::endl;
        std::cout << "\t\t" << r.dist_r1_3d_criticals[1] << std::endl;
        std::cout << "\tDominating criticals for r_2: " << std::endl;
        std::cout << "\t\t" << r.dist_r2_3d_criticals[0] << std::endl;
        std::cout << "\t\t" << r.dist_r2_3d_criticals[1] << std::endl;
        std::cout << "\tDominating criticals for r_3: " << std::endl;
        std::cout << "\t\t" << r.dist_r3_3d_criticals[0] << std::endl;
        std::cout << "\t\t" << r.dist_r3_3d_criticals[1] << std::endl;
    }
}

// The reference's split counts (tight_rectangle.cu:44-58); the environment
// variable CC_TIGHT_LAMBDA_MAX narrows the lambda range for short runs, and
// CC_TIGHT_GRID="la:r1,r2,r3,r4:g1,...,gk:s1,s2,s3,s4" replaces the split
// counts (initial lambda and radius splits, the lambda splits of the k
// refinement generations, their radius splits).
cc_tight_grid reference_grid() {
    cc_tight_grid g{};
    g.la_splits_init = 256;
    for (int k = 0; k < 4; ++k) g.r_splits_init[k] = 128;
    const int subdiv[11] = {1, 2, 2, 2, 2, 1, 2, 1, 2, 1, 2};
    g.num_generations = 11;
    for (int k = 0; k < 11; ++k) g.la_splits_gen[k] = subdiv[k];
    g.r_splits_gen[0] = 128;
    g.r_splits_gen[1] = 128;
    g.r_splits_gen[2] = 128;
    g.r_splits_gen[3] = 64;
    if (const char* e = std::getenv("CC_TIGHT_GRID")) {
        const std::vector<std::string> f = split_fields(e);
        if (f.size() != 4) throw std::runtime_error("CC_TIGHT_GRID: la:r1,r2,r3,r4:g1,...:s1,s2,s3,s4");
        parse_ints(f[0], &g.la_splits_init, 1);
        parse_ints(f[1], g.r_splits_init, 4);
        g.num_generations = f[2].empty() ? 0 : parse_ints(f[2], g.la_splits_gen, CC_MAX_GENERATIONS);
        parse_ints(f[3], g.r_splits_gen, 4);
    }
    return g;
}

}  // namespace dropin
}  // namespace circlecover

void circlecover::tight_rectangle::find_critical_intervals() {
    using namespace circlecover::dropin;
    begin_case("Critical intervals for rectangles (tight)");
    cc_handle* h = nullptr;
    check(nullptr, cc_create(&h, 0), "cc_create");
    const double dbl_max = 1.7976931348623157e308;
    double la_hi = 2.0898841580413818342;
    if (const char* e = std::getenv("CC_TIGHT_LAMBDA_MAX")) la_hi = std::strtod(e, nullptr);
    cc_tight_box root{{1.0, la_hi}, {{0.0, dbl_max}, {0.0, dbl_max}, {0.0, dbl_max}, {0.0, dbl_max}}};
    cc_tight_grid grid = reference_grid();

    std::cerr << "Initializing and refining - press Ctrl-C to interrupt and use best result achieved so far..." << std::endl;
    g_interrupts.store(0);
    g_active.store(h);
    void (*previous)(int) = std::signal(SIGINT, on_sigint);
    cc_tight_box* crit = nullptr;
    size_t n = 0;
    cc_prove_stats stats;
    // CC_TIGHT_CHECKPOINT=<file>: state written after every generation; an
    // existing file is resumed from
    const char* ckpt = std::getenv("CC_TIGHT_CHECKPOINT");
    int st;
    if (ckpt && *ckpt) {
        check(h, cc_set_checkpoint(h, ckpt), "cc_set_checkpoint");
        if (FILE* f = std::fopen(ckpt, "rb")) {
            std::fclose(f);
            std::cerr << "Resuming from " << ckpt << std::endl;
            st = cc_tight_resume(h, ckpt, &grid, 0, &crit, &n, &stats);
        } else {
            st = cc_tight_prove(h, &root, &grid, &crit, &n, &stats);
        }
    } else {
        st = cc_tight_prove(h, &root, &grid, &crit, &n, &stats);
    }
    std::signal(SIGINT, previous);
    g_active.store(nullptr);
    check(h, st, "cc_tight_prove");
    std::cerr << "Generations run: " << stats.generations_run << ", criticals: " << n << ", leaves: " << stats.leaf_evals
              << ", " << stats.seconds << " s" << std::endl;

    if (n) {
        cc_tight_summary_t summary;
        check(h, cc_tight_summary(h, crit, n, &summary), "cc_tight_summary");
        print_summary(summary);
    }
    cc_free(crit);
    cc_destroy(h);
    end_case();
}
