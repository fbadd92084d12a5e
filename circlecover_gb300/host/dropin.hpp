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
#include <vector>

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

// Comma-separated integers of one field of a split-count override
// ("a,b,c"); returns how many were read (at most `cap`).
inline int parse_ints(const std::string& field, int* out, int cap) {
    int n = 0;
    std::size_t pos = 0;
    while (pos < field.size() && n < cap) {
        std::size_t end = field.find(',', pos);
        if (end == std::string::npos) end = field.size();
        out[n++] = std::atoi(field.substr(pos, end - pos).c_str());
        pos = end + 1;
    }
    return n;
}

// Colon-separated fields of an override string.
inline std::vector<std::string> split_fields(const char* text) {
    std::vector<std::string> f;
    std::string s(text);
    std::size_t pos = 0;
    for (;;) {
        std::size_t end = s.find(':', pos);
        f.push_back(s.substr(pos, end == std::string::npos ? std::string::npos : end - pos));
        if (end == std::string::npos) break;
        pos = end + 1;
    }
    return f;
}

inline void check(cc_handle* h, int status, const char* what) {
    if (status != CC_OK && status != CC_ERR_INTERRUPTED) {
        throw std::runtime_error(std::string(what) + ": " + cc_status_str(status) + (h ? std::string(" (") + cc_last_error(h) + ")" : ""));
    }
}

}  // namespace dropin
}  // namespace circlecover
