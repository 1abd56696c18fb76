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
// ghost layer and the normal component is 0.  The field is stored as S
// (FP64, or its FP32 copy in the mixed-precision advection); the value is
// returned in the arithmetic type T of the caller.
template <typename T = double, typename S = double>
struct VelFPT {
    const S* v;
    Grid g;
    T scale;
    __device__ inline T operator()(int n, int i, int j, int k) const {
        i = wrapn(i, g.nx);
        j = wrapn(j, g.ny);
        const long long N = g.N;
        const S* c = v + n * N;
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
template <typename T = double, typename S = double>
struct CellFOT {
    const S* v;
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

// ---- FP64 decisions on the integer pipe.
// On this GPU every FP64 instruction -- DFMA, DADD, DMUL, and also the
// compares (DSETP) and min/max (DMNMX) -- issues at one sixty-fourth of the
// FP32 rate, while 64-bit integer compares and selects cost no FP64 issue
// slot.  Doubles that are not NaN order like their bit patterns read as
// sign-magnitude integers, so signs, comparisons, minima and maxima are taken
// on the bits.  Results equal the FP64 forms for every non-NaN operand, except
// that -0 orders below +0 (min/max may return the other zero).  NaN operands
// are not ordered like IEEE does; a NaN field still reaches the host through
// the arithmetic it enters and the residual / CFL maxima (imax_abs keeps it).
#ifdef __CUDACC__
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ double bitsd(long long b) { return __longlong_as_double(b); }
constexpr long long kMag = 0x7fffffffffffffffLL;
// signed integer with the order of the doubles
__device__ __forceinline__ long long okey(double x) {
    const long long b = dbits(x);
    return b ^ ((b >> 63) & kMag);
}
__device__ __forceinline__ bool igt0(double x) { return dbits(x) > 0; }   // x > 0
__device__ __forceinline__ bool ile0(double x) { return dbits(x) <= 0; }  // x <= 0
__device__ __forceinline__ bool ilt0(double x) { return okey(x) < -1; }   // x < 0 (-0 is not)
__device__ __forceinline__ bool ige0(double x) { return okey(x) >= -1; }  // x >= 0 (-0 is)
// ilt / imin / imax order -0 below +0 (okey(-0) = -1, okey(+0) = 0), where IEEE
// compares them equal: a +-0 tie goes to the signed zero's order, not to the
// first operand as fmin / fmax may
__device__ __forceinline__ bool ilt(double a, double b) { return okey(a) < okey(b); }
__device__ __forceinline__ double imin(double a, double b) { return okey(a) < okey(b) ? a : b; }
__device__ __forceinline__ double imax(double a, double b) { return okey(a) > okey(b) ? a : b; }
__device__ __forceinline__ double iabs(double x) { return bitsd(dbits(x) & kMag); }
// |x| < c for c > 0
__device__ __forceinline__ bool iabs_lt(double x, double c) { return (dbits(x) & kMag) < dbits(c); }
// |a| < |b|
__device__ __forceinline__ bool iabs_lt2(double a, double b) { return (dbits(a) & kMag) < (dbits(b) & kMag); }
// a and b non-zero with the same sign (a * b > 0 unless the product underflows)
__device__ __forceinline__ bool isame_sign(double a, double b) {
    return (dbits(a) ^ dbits(b)) >= 0 && (dbits(a) & kMag) != 0 && (dbits(b) & kMag) != 0;
}
// copysign(m, s) for m >= 0
__device__ __forceinline__ double isign(double m, double s) { return bitsd(dbits(m) | (dbits(s) & ~kMag)); }
// running max of |x| kept as bits: NaN patterns order above infinity, so a
// NaN operand survives to the host
__device__ __forceinline__ long long imax_abs(long long m, double x) {
    const long long b = dbits(x) & kMag;
    return b > m ? b : m;
}
#endif

}  // namespace ks
