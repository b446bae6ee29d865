// Minimal stand-in for the AMReX umbrella header, enough for the reference's
// header-only force kernels (src/chemistry/bmx_cell_interaction_K.H) to compile
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
namespace amrex {
using Real = double;
template <class T> using Vector = std::vector<T>;
}
#endif
