// Shared pieces of the drop-in host drivers (tight_rectangle.cpp,
// rectangle_size_bound.cpp): the reference's case banners, its interval text
// format, Ctrl-C forwarding to the library and status checks.
#pragma once

#include <atomic>
#include <csignal>
#include <cstdlib>
#include <iomanip>
#include <iostream>
#include <stdexcept>
#include <string>

#include "circlecover_gb300.h"

namespace circlecover {
namespace dropin {

static constexpr std::size_t kOutputWidth = 120;

// 120-column banner (reference: output_case.hpp:35-54)
inline void begin_case(const char* message) {
    std::string m(message);
    if (m.size() >= kOutputWidth - 2) {
        std::cout << m << std::endl;
        return;
    }
    std::size_t pre = (kOutputWidth - m.size() - 2) / 2;
    std::size_t post = kOutputWidth - m.size() - 2 - pre;
    std::cout << std::string(pre, '-') << ' ' << m << ' ' << std::string(post, '-') << std::endl;
}

inline void end_case() { std::cout << std::string(kOutputWidth, '-') << std::endl; }

// interval as "[lb, ub]", 19 significant digits, width 26 (reference: interval.hpp:294-303)
inline std::ostream& operator<<(std::ostream& o, const cc_iv& iv) {
    std::ios_base::fmtflags f = o.flags(std::ios::right);
    std::streamsize p = o.precision(19);
    o << '[' << std::setw(26) << iv.lb << ", " << std::setw(26) << iv.ub << ']';
    o.flags(f);
    o.precision(p);
    return o;
}

inline std::atomic<cc_handle*> g_active{nullptr};
inline std::atomic<int> g_interrupts{0};

extern "C" inline void on_sigint(int) {
    if (g_interrupts.fetch_add(1) > 0) std::_Exit(SIGINT);
    cc_handle* h = g_active.load();
    if (h) cc_interrupt(h);
}

inline void check(cc_handle* h, int status, const char* what) {
    if (status != CC_OK && status != CC_ERR_INTERRUPTED) {
        throw std::runtime_error(std::string(what) + ": " + cc_status_str(status) + (h ? std::string(" (") + cc_last_error(h) + ")" : ""));
    }
}

}  // namespace dropin
}  // namespace circlecover
