// ORACLE -- test infrastructure only.  CPU restatement of the OllinAxis-BiB
// evolution path used to check the GB300 library; never linked into it.
//
// Grid-function storage mirroring the reference: every grid function is a
// real(8) array (1-ghost:Nr, 1-ghost:Nz), column-major (r fastest)
// (generated allocatearrays.f90, prl/arrays.pl:86-111).
#pragma once
#include <cmath>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace oracle {

struct Arr {
    int g = 0, nr = 0, nz = 0, ld = 0;
    std::vector<double> v;
    Arr() {}
    Arr(int g_, int nr_, int nz_) : g(g_), nr(nr_), nz(nz_), ld(nr_ + g_), v((size_t)(nr_ + g_) * (nz_ + g_), 0.0) {}
    inline double& operator()(int i, int j) { return v[(size_t)(i - 1 + g) + (size_t)(j - 1 + g) * ld]; }
    inline double operator()(int i, int j) const { return v[(size_t)(i - 1 + g) + (size_t)(j - 1 + g) * ld]; }
};

// Boundary history (0:ghost-1, 1-ghost:Nz, 0:2) for r strips, and
// (1-ghost:Nr, 0:ghost-1, 0:2) for z strips (allocatearrays.f90).
struct Hist {
    int n0 = 0, n1 = 0;  // extents of the first two dimensions
    int lo1 = 0;         // lower bound of the second dimension (r strips) or first (z strips)
    std::vector<double> v;
};

// Integer powers as square-and-multiply from the most significant bit; the
// Fortran ``x**n`` of the reference evaluated by one fixed chain.
inline double p2(double x) { return x * x; }
inline double p3(double x) { return (x * x) * x; }
inline double p4(double x) { double a = x * x; return a * a; }
inline double p5(double x) { double a = x * x; a = a * a; return a * x; }
inline double p6(double x) { double a = x * x; a = a * x; return a * a; }
inline double p7(double x) { double a = x * x; a = a * x; a = a * a; return a * x; }
inline double p8(double x) { double a = x * x; a = a * a; return a * a; }

// Fortran nint: nearest integer, halves away from zero
inline double nint_(double x) { return std::round(x); }

}  // namespace oracle
