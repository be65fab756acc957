// Stand-in for pyre-journal's channel interface, which isce3 uses only to
// log (core/Spline2dInterpolator.cpp logs an out-of-range spline order).
// TEST INFRASTRUCTURE for the oracle's reference build (oracle/Makefile,
// target "ref"); messages are discarded.
#pragma once

#define __HERE__ 0

namespace pyre {
namespace journal {

struct located {};
inline located at(int) { return {}; }
struct newline_t {};
struct endl_t {};
constexpr newline_t newline{};
constexpr endl_t endl{};

class error_t {
public:
    explicit error_t(const char*) {}
    template <typename T>
    error_t& operator<<(const T&) { return *this; }
};
using warning_t = error_t;
using info_t = error_t;

}  // namespace journal
}  // namespace pyre
