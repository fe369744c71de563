// i2_dfvec.cuh -- small vectors, triangles and warp reductions in double-float (i2_dfloat.cuh),
// for the stages of the mixed form that compute in it (closed forms, potential tiers, adaptive
// potential).
#pragma once

#include "i2_device.cuh"
#include "i2_dfloat.cuh"

namespace i2 {

using df3 = V3<dfl>;
using TriD = TriT<dfl>;
using PanelJD = PanelJT<dfl>;
using FarCtxD = FarCtxT<dfl>;
using PotEdgeD = PotEdgeT<dfl>;

// ------------------------------------------------------------------ vector helpers
// dot product from exact partial products: the three high products are added error-free, the
// low-order terms (their rounding errors, the cross terms with the low parts, the additions'
// errors) in FP32 -- the error stays at about 2^-48 of the largest product, the precision the
// operands themselves carry, at about 40 FP32 operations instead of 64 for three products and
// two accurate additions.  Found by argument-dependent lookup ahead of the generic template.
__device__ __forceinline__ dfl dot(df3 a, df3 b)
{
    const dfl px = df_two_prod(a.x.hi, b.x.hi), py = df_two_prod(a.y.hi, b.y.hi), pz = df_two_prod(a.z.hi, b.z.hi);
    const dfl s1 = df_two_sum(px.hi, py.hi), s2 = df_two_sum(s1.hi, pz.hi);
    float lo = fmaf(a.x.lo, b.x.hi, a.x.hi * b.x.lo) + fmaf(a.y.lo, b.y.hi, a.y.hi * b.y.lo) + fmaf(a.z.lo, b.z.hi, a.z.hi * b.z.lo);
    lo += (px.lo + py.lo) + (pz.lo + (s1.lo + s2.lo));
    return df_two_sum(s2.hi, lo);
}

// a.y b.z - a.z b.y and the other two components, each as an exact difference of exact products
__device__ __forceinline__ dfl df_det2(dfl a, dfl b, dfl c, dfl d)  // a b - c d
{
    const dfl p = df_two_prod(a.hi, b.hi), q = df_two_prod(c.hi, d.hi);
    const dfl s = df_two_sum(p.hi, -q.hi);
    float lo = fmaf(a.lo, b.hi, a.hi * b.lo) - fmaf(c.lo, d.hi, c.hi * d.lo);
    lo += (p.lo - q.lo) + s.lo;
    return df_two_sum(s.hi, lo);
}

__device__ __forceinline__ df3 cross(df3 a, df3 b)
{
    return df3{df_det2(a.y, b.z, a.z, b.y), df_det2(a.z, b.x, a.x, b.z), df_det2(a.x, b.y, a.y, b.x)};
}

__device__ __forceinline__ dfl df_half(dfl x) { return dfl(0.5f * x.hi, 0.5f * x.lo); }
__device__ __forceinline__ df3 df_half(df3 a) { return df3{df_half(a.x), df_half(a.y), df_half(a.z)}; }

// the reference's child order (the FP64 child()), midpoints by exact halving
__device__ __forceinline__ TriD child_df(const TriD &t, int k)
{
    const df3 mbc = df_half(t.b + t.c), mca = df_half(t.c + t.a), mab = df_half(t.a + t.b);
    switch (k) {
    case 0: return TriD{mab, t.b, mbc};
    case 1: return TriD{mbc, t.c, mca};
    case 2: return TriD{mca, t.a, mab};
    default: return TriD{mbc, mca, mab};
    }
}

__device__ __forceinline__ TriD subcell_df(TriD t, int level, unsigned long long s)
{
    for (int l = level - 1; l >= 0; --l) t = child_df(t, (int)((s >> (2 * l)) & 3));
    return t;
}

__device__ __forceinline__ dfl warp_sum_df(dfl x)
{
    // the double-float sum is commutative, so every lane ends with the same value
    for (int off = 16; off > 0; off >>= 1) x = x + dfl(__shfl_xor_sync(0xffffffffu, x.hi, off), __shfl_xor_sync(0xffffffffu, x.lo, off));
    return x;
}

// a double-float value in a double's 8 bytes (the queue items' value slot), and back
__device__ __forceinline__ double df_pack(dfl v) { return __hiloint2double(__float_as_int(v.hi), __float_as_int(v.lo)); }
__device__ __forceinline__ dfl df_unpack(double d) { return dfl(__int_as_float(__double2hiint(d)), __int_as_float(__double2loint(d))); }

__device__ __forceinline__ df3 to_df(d3 a) { return df3{dfl(a.x), dfl(a.y), dfl(a.z)}; }
__device__ __forceinline__ TriD to_df(const Tri &t) { return TriD{to_df(t.a), to_df(t.b), to_df(t.c)}; }

__device__ __forceinline__ void tri_store_df(double *dst, const TriD &T)
{
    float *f = reinterpret_cast<float *>(dst);
    const dfl v[9] = {T.a.x, T.a.y, T.a.z, T.b.x, T.b.y, T.b.z, T.c.x, T.c.y, T.c.z};
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        f[2 * i] = v[i].hi;
        f[2 * i + 1] = v[i].lo;
    }
}

__device__ __forceinline__ TriD tri_load_df(const double *src)
{
    const float *f = reinterpret_cast<const float *>(src);
    dfl v[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) v[i] = dfl(f[2 * i], f[2 * i + 1]);
    return TriD{df3{v[0], v[1], v[2]}, df3{v[3], v[4], v[5]}, df3{v[6], v[7], v[8]}};
}

} // namespace i2
