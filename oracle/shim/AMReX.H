// Minimal stand-in for the AMReX umbrella header, enough for the reference's
// header-only kernels (src/chemistry/bmx_cell_interaction_K.H, bmx_chem_K.H) to compile
// as plain host C++. Oracle infrastructure only; never part of the product.
#ifndef BMXG_SHIM_AMREX_H
#define BMXG_SHIM_AMREX_H
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>
#define AMREX_GPU_HOST_DEVICE
#define AMREX_GPU_DEVICE
#define AMREX_GPU_HOST
#define AMREX_INLINE inline
#define AMREX_FORCE_INLINE inline
#include <cstdlib>
#include <iostream>  // the chemistry kernels print with std::cout
namespace amrex {
using Real = double;
template <class T> using Vector = std::vector<T>;
// bmx_chem_K.H's splitting and fusion kernels take a random engine; the
// harness hands them a fixed sequence of draws (u[0], u[1], ... in call
// order), and 0.5 once the sequence is used up or absent
struct RandomEngine {
    const double *u = nullptr;
    long n = 0;
    long *k = nullptr;
};
inline Real Random(RandomEngine const &e)
{
    if (!e.u || !e.k || *e.k >= e.n) return 0.5;
    return e.u[(*e.k)++];
}
inline void Abort(const char *msg) { std::fprintf(stderr, "%s\n", msg); std::abort(); }
}
#endif
