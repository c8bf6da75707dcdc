// Storage codecs for the distribution arrays.
//
//   Codec<double, double>, Codec<float, float>: plain values (FP64 / FP32 forms)
//   Codec<float, __half>, Codec<float, __nv_bfloat16>: 16-bit deviations from
//       the rest-state equilibrium, d_p = (f_p - w_p) / s_p, with one scale s_p
//       per population, and FP32 arithmetic (the mixed form): stage (a) decodes
//       and re-encodes; the flux kernel interpolates the stored deviations,
//       carries face values as f - w (dec_e) and updates in deviation units
//       (encode_dh), never forming f itself.
//       Stochastic rounding when sr_seed != 0 (the default of both forms;
//       config key rounding=nearest turns it off): hashed bits of (index, population, seed) are added below
//       the 16-bit mantissa of the float deviation before truncation (16 bits
//       for BF16, 13 for FP16), so the rounding error has zero mean and does
//       not bias time averages; the seed changes every step and the result
//       stays deterministic.  The step kernels hash the
//       cell once (cell_hash) and draw the population's bits from it with one
//       multiply by an odd constant (encode_dh), a bijection of the hash, so
//       each population's bits stay uniformly distributed.
#pragma once
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include "d3q19.cuh"

namespace dg {

template <class T, class S>
struct Codec {
    __device__ __forceinline__ T load(const S *a, long long idx, int) const { return T(a[idx]); }
    __device__ __forceinline__ T load_nc(const S *a, long long idx, int) const { return T(__ldg(a + idx)); }
    __device__ __forceinline__ T load_s(const S *a, int idx, int) const { return T(a[idx]); }
    __device__ __forceinline__ void store(S *a, long long idx, int, T v) const { a[idx] = S(v); }
    __device__ __forceinline__ unsigned cell_hash(long long) const { return 0u; }
    __device__ __forceinline__ S encode_h(int, T v, unsigned) const { return S(v); }
    __device__ __forceinline__ S encode_dh(int, T v, unsigned) const { return S(v); }
    __device__ __forceinline__ void store_h(S *a, long long idx, int p, T v, unsigned) const { store(a, idx, p, v); }
    // undecoded reads and the decode of a value affine in them (identity here)
    __device__ __forceinline__ T raw_nc(const S *a, long long idx) const { return T(__ldg(a + idx)); }
    __device__ __forceinline__ T raw_s(const S *a, int idx) const { return T(a[idx]); }
    __device__ __forceinline__ T raw(const S *a, long long idx) const { return T(a[idx]); }
    __device__ __forceinline__ T dec(int, T x) const { return x; }
    // the value less its rest-state equilibrium, as the flux kernels carry face
    // values (plain forms: the value itself, the rest state is not removed)
    __device__ __forceinline__ T dec_e(int, T x) const { return x; }
    __device__ __forceinline__ float2 dec_e2(int, int, float2 x) const { return x; }
    static constexpr bool deviation = false;
};

template <class S>
struct DevCodec {
    PopArr<float> w;  // rest-state equilibrium w_p (feq(rho=1, u=0))
    PopArr<float> s;  // scale s_p
    PopArr<float> is; // 1 / s_p
    unsigned sr_seed; // 0: round to nearest, else stochastic rounding with this seed
    static constexpr bool deviation = true;
};

// 32-bit integer mixer ("lowbias32", C. Wellons' hash-prospector, public domain)
__host__ __device__ __forceinline__ unsigned mix32(unsigned x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

template <>
struct Codec<float, __half> : DevCodec<__half> {
    __device__ __forceinline__ float load(const __half *a, long long idx, int p) const
    {
        return fmaf(s[p], __half2float(a[idx]), w[p]);
    }
    __device__ __forceinline__ float load_nc(const __half *a, long long idx, int p) const
    {
        return fmaf(s[p], __half2float(__ldg(a + idx)), w[p]);
    }
    __device__ __forceinline__ float load_s(const __half *a, int idx, int p) const
    {
        return fmaf(s[p], __half2float(a[idx]), w[p]);
    }
    // FP16 keeps 10 of the float's 23 fraction bits: r (13 random bits) added
    // to the float's bit pattern carries into the kept bits with probability
    // equal to the dropped fraction; the truncated float is then exact in FP16
    // (normal range; below 2^-14 the conversion truncates further, an error
    // under 2^-24 in deviation units).
    static __device__ __forceinline__ __half sr_half(float d, unsigned r)
    {
        const float t = __uint_as_float((__float_as_uint(d) + r) & ~0x1fffu);
        return __float2half_rz(t);
    }
    // deviation d rounded as the value stored at element idx (p: population)
    __device__ __forceinline__ __half encode_dev(long long idx, int p, float d) const
    {
        if (sr_seed == 0) return __float2half_rn(d);
        const unsigned r = mix32(unsigned(idx) * 19u + unsigned(p) + sr_seed * 0x9e3779b9u);
        return sr_half(d, r & 0x1fffu);
    }
    __device__ __forceinline__ void store(__half *a, long long idx, int p, float v) const
    {
        a[idx] = encode_dev(idx, p, (v - w[p]) * is[p]);
    }
    __device__ __forceinline__ unsigned cell_hash(long long cell) const
    {
        return sr_seed ? (mix32(unsigned(cell) ^ sr_seed) | 1u) : 0u;
    }
    // deviation d stored with the cell hash h (0: round to nearest)
    __device__ __forceinline__ __half encode_dh(int p, float d, unsigned h) const
    {
        if (h == 0u) return __float2half_rn(d);
        return sr_half(d, (h * (0x9e3779b1u + 0x6a09e66eu * unsigned(p))) >> 19);  // odd multiplier per p
    }
    __device__ __forceinline__ __half encode_h(int p, float v, unsigned h) const
    {
        return encode_dh(p, (v - w[p]) * is[p], h);
    }
    __device__ __forceinline__ void store_h(__half *a, long long idx, int p, float v, unsigned h) const
    {
        a[idx] = encode_h(p, v, h);
    }
    __device__ __forceinline__ float raw_nc(const __half *a, long long idx) const { return __half2float(__ldg(a + idx)); }
    __device__ __forceinline__ float raw_s(const __half *a, int idx) const { return __half2float(a[idx]); }
    __device__ __forceinline__ float dec(int p, float x) const { return fmaf(s[p], x, w[p]); }
    __device__ __forceinline__ float dec_e(int p, float x) const { return s[p] * x; }
    __device__ __forceinline__ float2 dec_e2(int p, int q, float2 x) const
    {
        return __fmul2_rn(make_float2(s[p], s[q]), x);
    }
    // dec and the deviation of encode_h for the populations p, q at once
    __device__ __forceinline__ float2 dec2(int p, int q, float2 x) const
    {
        return __ffma2_rn(make_float2(s[p], s[q]), x, make_float2(w[p], w[q]));
    }
    __device__ __forceinline__ float2 dev2(int p, int q, float2 v) const
    {
        return __fmul2_rn(__fadd2_rn(v, make_float2(-w[p], -w[q])), make_float2(is[p], is[q]));
    }
    __device__ __forceinline__ float raw(const __half *a, long long idx) const { return __half2float(a[idx]); }
};

template <>
struct Codec<float, __nv_bfloat16> : DevCodec<__nv_bfloat16> {
    __device__ __forceinline__ float load(const __nv_bfloat16 *a, long long idx, int p) const
    {
        return fmaf(s[p], __bfloat162float(a[idx]), w[p]);
    }
    __device__ __forceinline__ float load_nc(const __nv_bfloat16 *a, long long idx, int p) const
    {
        return fmaf(s[p], __bfloat162float(__ldg(a + idx)), w[p]);
    }
    __device__ __forceinline__ float load_s(const __nv_bfloat16 *a, int idx, int p) const
    {
        return fmaf(s[p], __bfloat162float(a[idx]), w[p]);
    }
    // deviation d rounded as the value stored at element idx (p: population)
    __device__ __forceinline__ __nv_bfloat16 encode_dev(long long idx, int p, float d) const
    {
        if (sr_seed == 0) return __float2bfloat16_rn(d);
        const unsigned r = mix32(unsigned(idx) * 19u + unsigned(p) + sr_seed * 0x9e3779b9u);
        const unsigned u = __float_as_uint(d) + (r & 0xffffu);  // magnitude rounds up with probability = fraction
        return __ushort_as_bfloat16((unsigned short)(u >> 16));
    }
    __device__ __forceinline__ void store(__nv_bfloat16 *a, long long idx, int p, float v) const
    {
        a[idx] = encode_dev(idx, p, (v - w[p]) * is[p]);
    }
    // per-cell hash of the step kernels (0: round to nearest)
    __device__ __forceinline__ unsigned cell_hash(long long cell) const
    {
        return sr_seed ? (mix32(unsigned(cell) ^ sr_seed) | 1u) : 0u;
    }
    // deviation d stored with the cell hash h (0: round to nearest)
    __device__ __forceinline__ __nv_bfloat16 encode_dh(int p, float d, unsigned h) const
    {
        if (h == 0u) return __float2bfloat16_rn(d);
        const unsigned r = (h * (0x9e3779b1u + 0x6a09e66eu * unsigned(p))) >> 16;  // odd multiplier per p
        return __ushort_as_bfloat16((unsigned short)((__float_as_uint(d) + r) >> 16));
    }
    __device__ __forceinline__ __nv_bfloat16 encode_h(int p, float v, unsigned h) const
    {
        return encode_dh(p, (v - w[p]) * is[p], h);
    }
    __device__ __forceinline__ void store_h(__nv_bfloat16 *a, long long idx, int p, float v, unsigned h) const
    {
        a[idx] = encode_h(p, v, h);
    }
    __device__ __forceinline__ float raw_nc(const __nv_bfloat16 *a, long long idx) const
    {
        return __bfloat162float(__ldg(a + idx));
    }
    __device__ __forceinline__ float raw_s(const __nv_bfloat16 *a, int idx) const { return __bfloat162float(a[idx]); }
    __device__ __forceinline__ float dec(int p, float x) const { return fmaf(s[p], x, w[p]); }
    __device__ __forceinline__ float dec_e(int p, float x) const { return s[p] * x; }
    __device__ __forceinline__ float2 dec_e2(int p, int q, float2 x) const
    {
        return __fmul2_rn(make_float2(s[p], s[q]), x);
    }
    // dec and the deviation of encode_h for the populations p, q at once
    __device__ __forceinline__ float2 dec2(int p, int q, float2 x) const
    {
        return __ffma2_rn(make_float2(s[p], s[q]), x, make_float2(w[p], w[q]));
    }
    __device__ __forceinline__ float2 dev2(int p, int q, float2 v) const
    {
        return __fmul2_rn(__fadd2_rn(v, make_float2(-w[p], -w[q])), make_float2(is[p], is[q]));
    }
    __device__ __forceinline__ float raw(const __nv_bfloat16 *a, long long idx) const { return __bfloat162float(a[idx]); }
};

}  // namespace dg
