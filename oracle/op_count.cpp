// op_count.cpp — operation counter of the oracle (test/measurement infrastructure).
//
// Compiles chem_oracle.c unchanged as C++ with every `double` replaced by a
// counting type, so each +, -, *, / and each math-library call the oracle
// executes is tallied. The counts of one chemistry step divided by the cells
// integrated give the algorithmic FP64 work per cell-step of the reference
// scheme (the numerator of the roofline figures of the benchmark).
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>

namespace opc {
enum { ADD, MUL, DIV, EXP, LOG, LOG10, POW, SQRT, TRIG, TANH, CMP, NCAT };
static thread_local unsigned long long cnt[NCAT];
}  // namespace opc

struct CD {
    double v;
    CD() = default;
    constexpr CD(double x) : v(x) {}
    constexpr CD(int x) : v((double)x) {}
    explicit operator int() const { return (int)v; }
    explicit operator double() const { return v; }
    friend CD operator+(CD a, CD b) { opc::cnt[opc::ADD]++; return CD(a.v + b.v); }
    friend CD operator-(CD a, CD b) { opc::cnt[opc::ADD]++; return CD(a.v - b.v); }
    friend CD operator*(CD a, CD b) { opc::cnt[opc::MUL]++; return CD(a.v * b.v); }
    friend CD operator/(CD a, CD b) { opc::cnt[opc::DIV]++; return CD(a.v / b.v); }
    friend CD operator-(CD a) { return CD(-a.v); }
    CD& operator+=(CD b) { return *this = *this + b; }
    CD& operator-=(CD b) { return *this = *this - b; }
    CD& operator*=(CD b) { return *this = *this * b; }
    CD& operator/=(CD b) { return *this = *this / b; }
    friend bool operator<(CD a, CD b) { opc::cnt[opc::CMP]++; return a.v < b.v; }
    friend bool operator<=(CD a, CD b) { opc::cnt[opc::CMP]++; return a.v <= b.v; }
    friend bool operator>(CD a, CD b) { opc::cnt[opc::CMP]++; return a.v > b.v; }
    friend bool operator>=(CD a, CD b) { opc::cnt[opc::CMP]++; return a.v >= b.v; }
    friend bool operator==(CD a, CD b) { return a.v == b.v; }
    friend bool operator!=(CD a, CD b) { return a.v != b.v; }
};
static_assert(sizeof(CD) == sizeof(double), "layout");

#define OPC_F1(name, cat) \
    static inline CD name(CD a) { opc::cnt[opc::cat]++; return CD(::name(a.v)); }
OPC_F1(exp, EXP)
OPC_F1(log, LOG)
OPC_F1(log10, LOG10)
OPC_F1(sqrt, SQRT)
OPC_F1(sin, TRIG)
OPC_F1(cos, TRIG)
OPC_F1(acos, TRIG)
OPC_F1(atan, TRIG)
OPC_F1(tanh, TANH)
static inline CD trunc(CD a) { return CD(::trunc(a.v)); }
static inline CD fabs(CD a) { return CD(::fabs(a.v)); }
static inline CD pow(CD a, CD b) { opc::cnt[opc::POW]++; return CD(::pow(a.v, b.v)); }
static inline CD fmax(CD a, CD b) { opc::cnt[opc::CMP]++; return CD(::fmax(a.v, b.v)); }
static inline CD fmin(CD a, CD b) { opc::cnt[opc::CMP]++; return CD(::fmin(a.v, b.v)); }

#define double CD
#include "chem_oracle.c"
#undef double

extern "C" {
// counts[NCAT]: add/sub, mul, div, exp, log, log10, pow, sqrt, trig, tanh, compare
void orc_count_reset(void) {
#pragma omp parallel
    { memset(opc::cnt, 0, sizeof(opc::cnt)); }
}
void orc_count_read(unsigned long long* out) {
    memset(out, 0, sizeof(unsigned long long) * opc::NCAT);
#pragma omp parallel
    {
#pragma omp critical
        for (int i = 0; i < opc::NCAT; i++) out[i] += opc::cnt[i];
    }
}
int orc_count_ncat(void) { return opc::NCAT; }
}
