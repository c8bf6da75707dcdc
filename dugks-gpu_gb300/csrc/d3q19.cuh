// D3Q19 discrete velocity set in the reference's population order
// (src/lbm_d3q19.cu:12-21): 0 rest; 1-6 +-x, +-y, +-z; 7-10 xy diagonals;
// 11-14 xz; 15-18 yz.  Written as constexpr functions so that fully unrolled
// population loops fold every velocity component to an immediate.
#pragma once

namespace dg {

constexpr int NPOP = 19;

__host__ __device__ constexpr int cx(int p)
{
    return (p == 1 || p == 7 || p == 9 || p == 11 || p == 13) ? 1
         : (p == 2 || p == 8 || p == 10 || p == 12 || p == 14) ? -1 : 0;
}
__host__ __device__ constexpr int cy(int p)
{
    return (p == 3 || p == 7 || p == 8 || p == 15 || p == 17) ? 1
         : (p == 4 || p == 9 || p == 10 || p == 16 || p == 18) ? -1 : 0;
}
__host__ __device__ constexpr int cz(int p)
{
    return (p == 5 || p == 11 || p == 12 || p == 15 || p == 16) ? 1
         : (p == 6 || p == 13 || p == 14 || p == 17 || p == 18) ? -1 : 0;
}
__host__ __device__ constexpr int cc(int axis, int p) { return axis == 0 ? cx(p) : axis == 1 ? cy(p) : cz(p); }

// Representative population of the class of p with the same c_x: 1 (c_x > 0),
// 2 (c_x < 0), 3 (c_x = 0).  The x-interpolation weight tables depend on p
// only through c_x, so reading them at the representative lets the compiler
// share one load per class.
__host__ __device__ constexpr int xrep(int p) { return cx(p) > 0 ? 1 : (cx(p) < 0 ? 2 : 3); }

// opposite population (src/lbm_d3q19.cu:15)
__host__ __device__ constexpr int opp(int p)
{
    return p == 0 ? 0 : (p <= 6 ? (p % 2 ? p + 1 : p - 1)
                                : (p <= 10 ? 17 - p : (p <= 14 ? 25 - p : 33 - p)));
}

// lattice weights 1/3, 1/18, 1/36 (src/lbm_d3q19.cu:17-19)
template <class T>
__host__ __device__ constexpr T weight(int p)
{
    return p == 0 ? T(1.0 / 3.0) : (p <= 6 ? T(1.0 / 18.0) : T(1.0 / 36.0));
}

// 19 per-population values with population 1 at an 8-byte boundary, so that
// each pair (2m-1, 2m) of the packed FP32x2 code is one aligned 8-byte word
template <class T>
struct alignas(8) PopArr {
    T pad_, v[NPOP];
    __host__ __device__ T &operator[](int p) { return v[p]; }
    __host__ __device__ const T &operator[](int p) const { return v[p]; }
};

// The 10 populations that cross a face normal to `axis` (c_axis != 0), in
// ascending order; the flux of a face is stored for these only.
__host__ __device__ constexpr int flux_pop(int axis, int s)
{
    // x: 1 2 7 8 9 10 11 12 13 14 ; y: 3 4 7 8 9 10 15 16 17 18 ; z: 5 6 11 12 13 14 15 16 17 18
    return axis == 0 ? (s < 2 ? 1 + s : 5 + s)
         : axis == 1 ? (s < 2 ? 3 + s : (s < 6 ? 5 + s : 9 + s))
                     : (s < 2 ? 5 + s : 9 + s);
}
// slot of population p in the flux list of `axis` (-1 if c_axis(p) == 0)
__host__ __device__ constexpr int flux_slot(int axis, int p)
{
    return axis == 0 ? (p == 1 || p == 2 ? p - 1 : (p >= 7 && p <= 14 ? p - 5 : -1))
         : axis == 1 ? (p == 3 || p == 4 ? p - 3 : (p >= 7 && p <= 10 ? p - 5 : (p >= 15 ? p - 9 : -1)))
                     : (p == 5 || p == 6 ? p - 5 : (p >= 11 ? p - 9 : -1));
}

}  // namespace dg
