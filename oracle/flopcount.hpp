// flopcount.hpp -- a counting scalar for exact operation counts of the oracle
// recursions (the algorithmic-flop figure of the roofline).
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cmath>
#include <cstdint>

namespace sbgo {

struct CReal {
    double v = 0;
    static inline thread_local int64_t n[6] = {};  // add, mul, div, sqrt, trig/tanh/pow, abs/compare
    CReal() = default;
    explicit CReal(double x) : v(x) {}
    static void reset() { for (auto& x : n) x = 0; }
    static void get(int64_t* out) { for (int i = 0; i < 6; ++i) out[i] = n[i]; }
};
inline CReal operator+(CReal a, CReal b) { ++CReal::n[0]; return CReal(a.v + b.v); }
inline CReal operator-(CReal a, CReal b) { ++CReal::n[0]; return CReal(a.v - b.v); }
inline CReal operator-(CReal a) { return CReal(-a.v); }
inline CReal operator*(CReal a, CReal b) { ++CReal::n[1]; return CReal(a.v * b.v); }
inline CReal operator/(CReal a, CReal b) { ++CReal::n[2]; return CReal(a.v / b.v); }
inline bool operator==(CReal a, CReal b) { ++CReal::n[5]; return a.v == b.v; }
inline bool operator>(CReal a, CReal b) { ++CReal::n[5]; return a.v > b.v; }
inline CReal sqrt(CReal a) { ++CReal::n[3]; return CReal(std::sqrt(a.v)); }
inline CReal sin(CReal a) { ++CReal::n[4]; return CReal(std::sin(a.v)); }
inline CReal cos(CReal a) { ++CReal::n[4]; return CReal(std::cos(a.v)); }
inline CReal abs(CReal a) { ++CReal::n[5]; return CReal(std::fabs(a.v)); }
inline CReal tanh(CReal a) { ++CReal::n[4]; return CReal(std::tanh(a.v)); }
inline CReal pow(CReal a, CReal b) { ++CReal::n[4]; return CReal(std::pow(a.v, b.v)); }
inline CReal min(CReal a, CReal b) { ++CReal::n[5]; return a.v < b.v ? a : b; }

}  // namespace sbgo
