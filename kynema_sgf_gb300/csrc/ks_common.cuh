// Shared device definitions: grid descriptor, index maps with periodic wrap,
// boundary-condition accessors and kernel declarations.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

namespace ks {

enum ZBC { ZPER = 0, ZSLIP = 1, ZWALLMODEL = 2 };

constexpr double kSmallVel = 1.0e-8;  // AMReX-Hydro small_vel

// Uniform single-box grid.  x and y are periodic; z is periodic (zper = 1) or
// bounded by a slip wall / wall-model wall at each end.
struct Grid {
    int nx, ny, nz;
    int zper;
    int zlo, zhi;
    double dx, dy, dz;
    double idx, idy, idz;  // 1/dx, 1/dy, 1/dz (FP64 division is expensive on this GPU)
    long long N;    // cells
    long long NFz;  // z faces stored: nx*ny*(nz+1)
};

__host__ __device__ inline long long cidx(const Grid& g, int i, int j, int k) {
    return ((long long)k * g.ny + j) * g.nx + i;
}
__host__ __device__ inline int wrapn(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
__host__ __device__ inline double hd(const Grid& g, int d) { return d == 0 ? g.dx : (d == 1 ? g.dy : g.dz); }
__host__ __device__ inline double ihd(const Grid& g, int d) { return d == 0 ? g.idx : (d == 1 ? g.idy : g.idz); }
__host__ __device__ inline int nd(const Grid& g, int d) { return d == 0 ? g.nx : (d == 1 ? g.ny : g.nz); }
__host__ __device__ inline int nzfaces(const Grid& g) { return g.zper ? g.nz : g.nz + 1; }

// Face arrays: x and y faces use the cell index of the cell on their high
// side (N entries, periodic); z faces use nx*ny*(nz+1) storage with layer k
// at k-1/2 (walls) or wrap into [0,nz) (periodic).
__host__ __device__ inline long long fidx(const Grid& g, int d, int i, int j, int k) {
    i = wrapn(i, g.nx);
    j = wrapn(j, g.ny);
    if (d != 2 || g.zper) k = wrapn(k, g.nz);
    return cidx(g, i, j, k);
}

// Cell-centred velocity (or rho*velocity) with fill-patch ghost values:
// periodic wrap in x, y (and z); at walls the tangential components take the
// high-order extrapolation to the face, (15 q0 - 10 q1 + 3 q2)/8, in every
// ghost layer and the normal component is 0.  The stored field is FP64; the
// value is returned in the arithmetic type T of the caller.
template <typename T = double>
struct VelFPT {
    const double* v;
    Grid g;
    T scale;
    __device__ inline T operator()(int n, int i, int j, int k) const {
        i = wrapn(i, g.nx);
        j = wrapn(j, g.ny);
        const long long N = g.N;
        const double* c = v + n * N;
        if (g.zper) return scale * (T)c[cidx(g, i, j, wrapn(k, g.nz))];
        if (k < 0) {
            if (n == 2) return T(0);
            const T q0 = (T)c[cidx(g, i, j, 0)], q1 = (T)c[cidx(g, i, j, 1)], q2 = (T)c[cidx(g, i, j, 2)];
            return scale * (T(0.125) * (T(15) * q0 - T(10) * q1 + T(3) * q2));
        }
        if (k >= g.nz) {
            if (n == 2) return T(0);
            const int t = g.nz - 1;
            const T q0 = (T)c[cidx(g, i, j, t)], q1 = (T)c[cidx(g, i, j, t - 1)], q2 = (T)c[cidx(g, i, j, t - 2)];
            return scale * (T(0.125) * (T(15) * q0 - T(10) * q1 + T(3) * q2));
        }
        return scale * (T)c[cidx(g, i, j, k)];
    }
};
using VelFP = VelFPT<double>;

// Cell field with first-order extrapolation ghosts in z (forces, viscosity).
template <typename T = double>
struct CellFOT {
    const double* v;
    Grid g;
    __device__ inline T operator()(int n, int i, int j, int k) const {
        i = wrapn(i, g.nx);
        j = wrapn(j, g.ny);
        if (g.zper) k = wrapn(k, g.nz);
        else k = k < 0 ? 0 : (k >= g.nz ? g.nz - 1 : k);
        return (T)v[n * g.N + cidx(g, i, j, k)];
    }
};
using CellFO = CellFOT<double>;

inline unsigned nblocks(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// max that keeps a NaN operand (fmax drops it): a non-finite residual or CFL
// maximum must reach the host's finiteness checks
__host__ __device__ inline double nmax(double a, double b) { return (a != a || b != b) ? a + b : (a > b ? a : b); }

}  // namespace ks
