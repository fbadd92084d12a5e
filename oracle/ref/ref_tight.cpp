/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * C entry points over the REFERENCE's own tight-rectangle criteria, compiled
 * for the host with ref_shim.h (see Makefile).  Only the driver loops, which
 * the reference writes as CUDA kernels, are restated (tight_driver.hpp and
 * the per-box evaluator below); every criterion call goes to the reference's
 * unmodified code.
 */
#include <csetjmp>
#include <cstdarg>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "tight_rectangle/strategies.cuh"
#include "../tight_driver.hpp"

using circlecover::IV;
namespace tr = circlecover::tight_rectangle;

/* ------------------------------------------------ shim runtime support */
CC_HOST_TLS unsigned long long cc_shim_op_count = 0;
static CC_HOST_TLS jmp_buf* cc_ref_trap_target = nullptr;
static CC_HOST_TLS uint32_t cc_ref_trapped = 0;
static CC_HOST_TLS unsigned long long cc_ref_printf_count = 0;

void algcuda::trap() noexcept {
    cc_ref_trapped = 1;
    if (cc_ref_trap_target) longjmp(*cc_ref_trap_target, 1);
    std::abort();
}

/* run f(ctx); a reference trap() inside it lands here: the call counts as
   "not certified" and *trapped is set */
bool cc_ref_guarded_call(bool (*f)(void*), void* ctx, uint32_t* trapped) {
    jmp_buf env;
    jmp_buf* prev = cc_ref_trap_target;
    uint32_t before = cc_ref_trapped;
    cc_ref_trapped = 0;
    cc_ref_trap_target = &env;
    bool r = false;
    if (setjmp(env) == 0) {
        r = f(ctx);
    } else {
        r = false;
    }
    cc_ref_trap_target = prev;
    *trapped = cc_ref_trapped;
    cc_ref_trapped = before | cc_ref_trapped;
    return r;
}

extern "C" int cc_ref_printf(const char* fmt, ...) {
    ++cc_ref_printf_count;
    if (std::getenv("CC_REF_PRINTF")) {
        va_list ap;
        va_start(ap, fmt);
        int r = std::vfprintf(stderr, fmt, ap);
        va_end(ap);
        return r;
    }
    return 0;
}

/* --------------------- restated driver helpers (tight_rectangle.cu:72-102) */
static IV ref_r1_range(IV la) {
    double f = __ddiv_rd(tr::critical_ratio(la).get_lb(), circlecover::rectangle_size_bound::critical_ratio);
    if (f <= 1.0) f = 1.0;
    double lb = __dmul_rd(circlecover::rectangle_size_bound::ub_disk_weight, f);
    double ub = __dmul_ru(0.25, __dadd_ru(1.0, __dmul_ru(la.get_ub(), la.get_ub())));
    return {lb, ub};
}

/* adapter for tight_driver.hpp */
struct RefCriteria {
    using V = IV;
    static V make(double l, double u) { return V(l, u); }
    static double lo(const V& v) { return v.get_lb(); }
    static double hi(const V& v) { return v.get_ub(); }
    static V sub(const V& a, const V& b) { return a - b; }
    static void tighten_lb(V& v, double x) { v.tighten_lb(x); }
    static void do_join(V& a, const V& b) { a.do_join(b); }
    static V intersect(const V& a, const V& b) { return a.intersect(b); }
    static bool empty(const V& v) { return v.empty(); }
    static V subinterval(const V& v, int i, int n) { return circlecover::get_subinterval(v, i, n); }
    static V required_weight(const V& la) { return tr::required_weight_for(la); }
    static V r1_range(const V& la) { return ref_r1_range(la); }
    /* r2..r4 ranges take the precomputed weight; the reference recomputes
       required_weight_for(la) inside each (tight_rectangle.cu:83-102), same bits */
    static V r2_range(const V& w, const V& r1) {
        double u2 = (w - r1).get_ub();
        return {0.0, r1.get_ub() < u2 ? r1.get_ub() : u2};
    }
    static V r3_range(const V& w, const V& r1, const V& r2) {
        double u2 = (w - r1 - r2).get_ub();
        return {0.0, r2.get_ub() < u2 ? r2.get_ub() : u2};
    }
    static V r4_range(const V& w, const V& r1, const V& r2, const V& r3) {
        double u2 = (w - r1 - r2 - r3).get_ub();
        return {0.0, r3.get_ub() < u2 ? r3.get_ub() : u2};
    }
    static bool r1_strategies(const V& la, const V& r1, double ub) { return guarded([&] { return tr::r1_strategies(la, r1, ub); }); }
    static bool r1_r2_strategies(const V& la, const V& r1, const V& r2, double ub) {
        return guarded([&] { return tr::r1_r2_strategies(la, r1, r2, ub); });
    }
    static bool r1_r2_r3_strategies(const V& la, const V& r1, const V& r2, const V& r3, double ub) {
        return guarded([&] { return tr::r1_r2_r3_strategies(la, r1, r2, r3, ub); });
    }
    template <class B>
    static tr::Variables vars(const B& b) {
        tr::Variables v;
        v.la = b.la;
        for (int k = 0; k < 4; ++k) v.radii[k] = b.r[k];
        return v;
    }
    template <class B>
    static bool two_by_two(const B& b, const V& R) { tr::Variables v = vars(b); return guarded([&] { return tr::two_by_two_strategies(v, R); }); }
    template <class B>
    static bool r1_r2_r3_leaf(const B& b, const V& R4) { tr::Variables v = vars(b); return guarded([&] { return tr::r1_r2_r3_strategies(v, R4); }); }
    template <class B>
    static bool gaps(const B& b, const V& R) { tr::Variables v = vars(b); return guarded([&] { return tr::r1_r2_large_r3_r4_gaps_strategy(v, R); }); }
    static uint32_t trapped() { return cc_ref_trapped; }
    static void clear_trap() { cc_ref_trapped = 0; }

    /* run one criterion; a reference trap() lands here and counts as "not certified" */
    template <class F>
    static bool guarded(F f) {
        jmp_buf env;
        jmp_buf* prev = cc_ref_trap_target;
        cc_ref_trap_target = &env;
        bool r = false;
        if (setjmp(env) == 0) {
            r = f();
        } else {
            r = false;
        }
        cc_ref_trap_target = prev;
        return r;
    }
};

using Driver = cc_oracle::TightDriver<RefCriteria>;

static IV to_iv(const cc_iv& x) { return IV(x.lb, x.ub); }
static cc_iv from_iv(const IV& x) { return cc_iv{x.get_lb(), x.get_ub()}; }

/* the per-box verdict mask (CC_TV_*) at the reference leaf's arguments */
static uint32_t eval_one(const cc_tight_box& in) {
    cc_ref_trapped = 0;
    IV la = to_iv(in.la), r1 = to_iv(in.r[0]), r2 = to_iv(in.r[1]), r3 = to_iv(in.r[2]), r4 = to_iv(in.r[3]);
    IV weight = tr::required_weight_for(la);
    uint32_t m = 0;
    if (RefCriteria::r1_strategies(la, r1, r2.get_ub())) m |= CC_TV_R1;
    if (RefCriteria::r1_r2_strategies(la, r1, r2, r3.get_ub())) m |= CC_TV_R1R2;
    if (RefCriteria::r1_r2_r3_strategies(la, r1, r2, r3, r4.get_ub())) m |= CC_TV_R1R2R3;
    IV R4 = weight - r1 - r2 - r3;
    R4.tighten_lb(0.0);
    tr::Variables v{la, {r1, r2, r3, r4}};
    v.radii[2].tighten_lb(v.radii[3].get_lb());
    v.radii[1].tighten_lb(v.radii[2].get_lb());
    v.radii[0].tighten_lb(v.radii[1].get_lb());
    IV R = weight - v.radii[0] - v.radii[1] - v.radii[2] - v.radii[3];
    R.tighten_lb(0.0);
    if (RefCriteria::guarded([&] { return tr::two_by_two_strategies(v, R); })) m |= CC_TV_TWO_BY_TWO;
    if (RefCriteria::guarded([&] { return tr::r1_r2_r3_strategies(v, R4); })) m |= CC_TV_R1R2R3_LEAF;
    if (RefCriteria::guarded([&] { return tr::r1_r2_large_r3_r4_gaps_strategy(v, R); })) m |= CC_TV_GAPS;
    if (R4.empty() || R.empty()) m |= CC_TV_R_EMPTY;
    if (cc_ref_trapped) m |= CC_TV_TRAPPED;
    return m;
}

template <class F>
static void parallel_for(size_t n, int threads, F f) {
    if (threads <= 1 || n < 1024) {
        f(0, n, 0);
        return;
    }
    std::vector<std::thread> pool;
    size_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        size_t b = t * chunk, e = b + chunk < n ? b + chunk : n;
        if (b >= e) break;
        pool.emplace_back(f, b, e, t);
    }
    for (auto& th : pool) th.join();
}

extern "C" {

/* masks[i] = verdict mask of boxes[i]; ops (optional) = primitive FP64
 * directed-rounding operations executed for box i */
int ccref_tight_eval(const cc_tight_box* boxes, size_t n, uint32_t* masks, uint64_t* ops, int threads) {
    parallel_for(n, threads, [&](size_t b, size_t e, int) {
        for (size_t i = b; i < e; ++i) {
            unsigned long long before = cc_shim_op_count;
            masks[i] = eval_one(boxes[i]);
            if (ops) ops[i] = cc_shim_op_count - before;
        }
    });
    return 0;
}

unsigned long long ccref_op_count(void) { return cc_shim_op_count; }

/* Restated reference driver.  Criticals are returned in a malloc'd array. */
int ccref_tight_prove(const cc_tight_box* root, const cc_tight_grid* grid, int threads, cc_tight_box** out, size_t* n_out,
                      cc_prove_stats* stats) {
    Driver::Box r{to_iv(root->la), {to_iv(root->r[0]), to_iv(root->r[1]), to_iv(root->r[2]), to_iv(root->r[3])}};
    Driver::Result res = Driver::prove(r, *grid, threads);
    *n_out = res.criticals.size();
    *out = (cc_tight_box*)std::malloc(sizeof(cc_tight_box) * (res.criticals.size() + 1));
    for (size_t i = 0; i < res.criticals.size(); ++i) {
        (*out)[i].la = from_iv(res.criticals[i].la);
        for (int k = 0; k < 4; ++k) (*out)[i].r[k] = from_iv(res.criticals[i].r[k]);
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        std::memcpy(stats->counts, res.trace.counts, sizeof(stats->counts));
        stats->digest = res.trace.digest;
        stats->leaf_evals = res.trace.leaf_evals;
        stats->trapped_leaves = res.trapped_leaves;
        for (size_t g = 0; g < res.gen_sizes.size() && g <= CC_MAX_GENERATIONS; ++g) stats->gen_sizes[g] = res.gen_sizes[g];
        stats->generations_run = res.generations_run;
    }
    return 0;
}

/* One generation of the restated driver over the tasks [lo, hi) (task =
 * parent index * la_splits + lambda piece), on the reference's own criteria:
 * the task-range oracle of the full proof's generations.  Criticals in task
 * order, merged per task; stats as ccref_tight_prove (gen_sizes[0] = count). */
int ccref_tight_generation(const cc_tight_box* parents, size_t n, int la_splits, const int* splits, uint64_t lo,
                           uint64_t hi, int threads, cc_tight_box** out, size_t* n_out, cc_prove_stats* stats) {
    std::vector<Driver::Box> in(n);
    for (size_t i = 0; i < n; ++i)
        in[i] = Driver::Box{to_iv(parents[i].la), {to_iv(parents[i].r[0]), to_iv(parents[i].r[1]),
                                                   to_iv(parents[i].r[2]), to_iv(parents[i].r[3])}};
    std::vector<Driver::Box> res;
    cc_oracle::Trace tr;
    tr.clear();
    uint64_t trapped = 0;
    Driver::generation(in, la_splits, splits, threads, res, tr, trapped, lo, hi);
    *n_out = res.size();
    *out = (cc_tight_box*)std::malloc(sizeof(cc_tight_box) * (res.size() + 1));
    for (size_t i = 0; i < res.size(); ++i) {
        (*out)[i].la = from_iv(res[i].la);
        for (int k = 0; k < 4; ++k) (*out)[i].r[k] = from_iv(res[i].r[k]);
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        std::memcpy(stats->counts, tr.counts, sizeof(stats->counts));
        stats->digest = tr.digest;
        stats->leaf_evals = tr.leaf_evals;
        stats->trapped_leaves = trapped;
        stats->gen_sizes[0] = res.size();
    }
    return 0;
}

void ccref_free(void* p) { std::free(p); }

/* single criteria, for targeted tests */
double ccref_tight_critical_ratio(double lo, double hi, double* out_hi) {
    IV c = tr::critical_ratio(IV(lo, hi));
    *out_hi = c.get_ub();
    return c.get_lb();
}
double ccref_two_disks_maximize_height(double r1lo, double r1hi, double r2lo, double r2hi, double ub_w) {
    return circlecover::rectangle_size_bound::two_disks_maximize_height(IV(r1lo, r1hi), IV(r2lo, r2hi), ub_w);
}
int ccref_tight_can_recurse(double w, double h, double largest, double weight) {
    return tr::can_recurse(w, h, largest, weight) ? 1 : 0;
}

/* Max_distances of a critical set: a restatement of the reference's
 * kernel_compute_distance_from_theoretical_worst_cases
 * (tight_rectangle/tight_rectangle.cu:343-456; a one-thread CUDA kernel
 * there) on the reference's own interval type and required_weight_for.
 * Deviation: the reference starts S1/h2/S3 from uninitialised device memory
 * and only overwrites them at the first box whose pocket width exceeds the
 * running one while that is negative; they start at zero here. */
static cc_iv civ(const IV& x) { return cc_iv{x.get_lb(), x.get_ub()}; }
static IV fiv(const cc_iv& x) { return IV(x.lb, x.ub); }
static cc_tight_box cbox(const tr::Variables& v) {
    cc_tight_box b;
    b.la = civ(v.la);
    for (int k = 0; k < 4; ++k) b.r[k] = civ(v.radii[k]);
    return b;
}

void ccref_tight_summary(const cc_tight_box* crit, size_t n, cc_tight_summary_t* out) {
    cc_tight_summary_t o;
    std::memset(&o, 0, sizeof(o));
    o.la_range_3d = cc_iv{1.0, 1.0};
    o.la_range_2d = cc_iv{2.0, 2.0};
    o.pocket_width_3d = -1.0;
    o.lb_h1_2d = 1.0;
    o.ub_la_by_S1 = 1.0;
    for (size_t i = 0; i < n; ++i) {
        tr::Variables v;
        v.la = fiv(crit[i].la);
        for (int k = 0; k < 4; ++k) v.radii[k] = fiv(crit[i].r[k]);
        auto track = [&](cc_iv& acc, const IV& d, cc_tight_box* dom) {
            if (d.get_lb() < acc.lb) dom[0] = cbox(v);
            if (d.get_ub() > acc.ub) dom[1] = cbox(v);
        };
        if (v.radii[2].get_ub() < 0.1) {
            o.have_range_2d = 1;
            IV lr = fiv(o.la_range_2d);
            lr.do_join(v.la);
            o.la_range_2d = civ(lr);
            IV r1_t = 0.25 * (v.la.square() + 1.0);
            IV r2_t{0.25, 0.25};
            IV d1 = v.radii[0] - r1_t, d2 = v.radii[1] - r2_t;
            track(o.dist_r1_2d, d1, o.dist_r1_2d_criticals);
            IV j1 = fiv(o.dist_r1_2d);
            j1.do_join(d1);
            o.dist_r1_2d = civ(j1);
            track(o.dist_r2_2d, d2, o.dist_r2_2d_criticals);
            IV j2 = fiv(o.dist_r2_2d);
            j2.do_join(d2);
            o.dist_r2_2d = civ(j2);
            IV R3 = tr::required_weight_for(v.la) - v.radii[0] - v.radii[1];
            if (R3.get_ub() > o.ub_R3_2d) o.ub_R3_2d = R3.get_ub();
            double lb_S1 = __dmul_rd(2.0, __dsqrt_rd(__dadd_rd(v.radii[0].get_lb(), -0.25)));
            double la_by_S1 = __ddiv_ru(v.la.get_ub(), lb_S1);
            if (la_by_S1 > o.ub_la_by_S1) o.ub_la_by_S1 = la_by_S1;
            double t = __dadd_ru(v.la.get_ub(), -__dmul_rd(0.5, lb_S1));
            double lb_h1 = __dmul_rd(2.0, __dsqrt_rd(__dadd_rd(v.radii[0].get_lb(), -__dmul_ru(t, t))));
            if (lb_h1 < o.lb_h1_2d) o.lb_h1_2d = lb_h1;
        } else {
            o.have_range_3d = 1;
            IV lr = fiv(o.la_range_3d);
            lr.do_join(v.la);
            o.la_range_3d = civ(lr);
            IV la2 = v.la.square();
            IV la4 = la2.square();
            IV theory = (16.0 * la4 + 40.0 * la2 + 9.0) / (256.0 * la2);
            IV d1 = v.radii[0] - theory, d2 = v.radii[1] - theory, d3 = v.radii[2] - theory;
            track(o.dist_r1_3d, d1, o.dist_r1_3d_criticals);
            track(o.dist_r2_3d, d2, o.dist_r2_3d_criticals);
            track(o.dist_r3_3d, d3, o.dist_r3_3d_criticals);
            IV j1 = fiv(o.dist_r1_3d), j2 = fiv(o.dist_r2_3d), j3 = fiv(o.dist_r3_3d);
            j1.do_join(d1);
            j2.do_join(d2);
            j3.do_join(d3);
            o.dist_r1_3d = civ(j1);
            o.dist_r2_3d = civ(j2);
            o.dist_r3_3d = civ(j3);
            IV R4 = tr::required_weight_for(v.la) - v.radii[0] - v.radii[1] - v.radii[2];
            if (R4.get_ub() > o.ub_R4_3d) o.ub_R4_3d = R4.get_ub();
            uint32_t trapped = 0;
            struct Ctx {
                const tr::Variables* v;
                IV S1, h2, S3;
            } cx{&v, IV(0.0, 0.0), IV(0.0, 0.0), IV(0.0, 0.0)};
            // the square roots trap on a negative lower bound (interval.cuh:339-346)
            cc_ref_guarded_call([](void* p) {
                Ctx& c = *(Ctx*)p;
                c.S1 = sqrt(4.0 * c.v->radii[0] - 1.0);
                c.h2 = sqrt(4.0 * c.v->radii[1] - (c.v->la - c.S1).square());
                c.S3 = sqrt(4.0 * c.v->radii[2] - (1.0 - c.h2).square());
                return true;
            }, &cx, &trapped);
            double pocket = (v.la - cx.S1 - cx.S3).get_ub();
            if (pocket > o.pocket_width_3d) {
                if (o.pocket_width_3d < 0.0) {
                    o.S1 = civ(cx.S1);
                    o.h2 = civ(cx.h2);
                    o.S3 = civ(cx.S3);
                }
                o.pocket_width_3d = pocket;
            }
            IV a = fiv(o.S1), c = fiv(o.h2), e = fiv(o.S3);
            a.do_join(cx.S1);
            c.do_join(cx.h2);
            e.do_join(cx.S3);
            o.S1 = civ(a);
            o.h2 = civ(c);
            o.S3 = civ(e);
        }
    }
    *out = o;
}

/* algcuda::Interval<double> * double (interval.cuh:185-197), for the
 * interval-times-scalar rounding test */
void ccref_iv_mul_scalar(double lo, double hi, double s, double* out) {
    IV r = IV(lo, hi) * s;
    out[0] = r.get_lb();
    out[1] = r.get_ub();
}

}  // extern "C"
