// f3d_numtypes.hpp — scalar types the oracle templates are instantiated on.
//
// TEST INFRASTRUCTURE ONLY.
//  Dual    : forward-mode dual number (value, tangent) for JVPs of the oracle. Branches
//            (abs, max, minmod, the hybrid-scheme switch) follow the value, so the JVP is
//            the derivative of the branch that the value takes; d|x|/dx is +1 at x = 0.
//  Counted : a double that counts every floating-point operation applied to it, for the
//            algorithmic operation count of one RHS evaluation.
#pragma once
#include <cmath>

namespace f3do {

struct Dual {
    double v, d;
    Dual(double value = 0.0, double tangent = 0.0) : v(value), d(tangent) {}
    friend Dual operator+(const Dual& a, const Dual& b) { return Dual(a.v + b.v, a.d + b.d); }
    friend Dual operator-(const Dual& a, const Dual& b) { return Dual(a.v - b.v, a.d - b.d); }
    friend Dual operator*(const Dual& a, const Dual& b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
    friend Dual operator/(const Dual& a, const Dual& b) {
        double q = a.v / b.v;
        return Dual(q, (a.d - q * b.d) / b.v);
    }
    friend Dual operator-(const Dual& a) { return Dual(-a.v, -a.d); }
    Dual& operator+=(const Dual& b) { v += b.v; d += b.d; return *this; }
    Dual& operator-=(const Dual& b) { v -= b.v; d -= b.d; return *this; }
    Dual& operator*=(const Dual& b) { *this = *this * b; return *this; }
    friend bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
    friend bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
    friend bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
    friend bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
    friend bool operator!=(const Dual& a, const Dual& b) { return a.v != b.v; }
    friend bool operator==(const Dual& a, const Dual& b) { return a.v == b.v; }
    friend Dual abs(const Dual& a) { return a.v >= 0.0 ? a : -a; }
    friend Dual cbrt(const Dual& a) {
        const double r = std::cbrt(a.v);
        return Dual(r, a.d / (3.0 * r * r));
    }
    friend Dual sqrt(const Dual& a) {
        double s = std::sqrt(a.v);
        return Dual(s, a.d / (2.0 * s));
    }
    // a^e for a constant exponent e
    friend Dual pow(const Dual& a, const Dual& e) {
        const double r = std::pow(a.v, e.v);
        return Dual(r, e.v * std::pow(a.v, e.v - 1.0) * a.d);
    }
};

// Operation counters (single-threaded use: the counting entry point runs on one thread).
enum { OPC_ADD = 0, OPC_MUL = 1, OPC_DIV = 2, OPC_SQRT = 3, OPC_CMP = 4, OPC_N = 5 };
inline double* opcount_table() {
    static double t[OPC_N] = {0, 0, 0, 0, 0};
    return t;
}
inline void opcount_reset() {
    for (int i = 0; i < OPC_N; i++) opcount_table()[i] = 0;
}
inline void opcount_read(double* out) {
    for (int i = 0; i < OPC_N; i++) out[i] = opcount_table()[i];
}

struct Counted {
    double v;
    Counted(double value = 0.0) : v(value) {}
    static void tick(int c) { opcount_table()[c] += 1.0; }
    friend Counted operator+(const Counted& a, const Counted& b) { tick(OPC_ADD); return Counted(a.v + b.v); }
    friend Counted operator-(const Counted& a, const Counted& b) { tick(OPC_ADD); return Counted(a.v - b.v); }
    friend Counted operator*(const Counted& a, const Counted& b) { tick(OPC_MUL); return Counted(a.v * b.v); }
    friend Counted operator/(const Counted& a, const Counted& b) { tick(OPC_DIV); return Counted(a.v / b.v); }
    friend Counted operator-(const Counted& a) { return Counted(-a.v); }
    Counted& operator+=(const Counted& b) { tick(OPC_ADD); v += b.v; return *this; }
    Counted& operator-=(const Counted& b) { tick(OPC_ADD); v -= b.v; return *this; }
    Counted& operator*=(const Counted& b) { tick(OPC_MUL); v *= b.v; return *this; }
    friend bool operator<(const Counted& a, const Counted& b) { tick(OPC_CMP); return a.v < b.v; }
    friend bool operator>(const Counted& a, const Counted& b) { tick(OPC_CMP); return a.v > b.v; }
    friend bool operator<=(const Counted& a, const Counted& b) { tick(OPC_CMP); return a.v <= b.v; }
    friend bool operator>=(const Counted& a, const Counted& b) { tick(OPC_CMP); return a.v >= b.v; }
    friend bool operator!=(const Counted& a, const Counted& b) { return a.v != b.v; }
    friend bool operator==(const Counted& a, const Counted& b) { return a.v == b.v; }
    friend Counted abs(const Counted& a) { tick(OPC_CMP); return Counted(std::fabs(a.v)); }
    friend Counted sqrt(const Counted& a) { tick(OPC_SQRT); return Counted(std::sqrt(a.v)); }
    friend Counted cbrt(const Counted& a) { tick(OPC_SQRT); return Counted(std::cbrt(a.v)); }
    friend Counted pow(const Counted& a, const Counted& e) { tick(OPC_SQRT); return Counted(std::pow(a.v, e.v)); }
};

}  // namespace f3do
