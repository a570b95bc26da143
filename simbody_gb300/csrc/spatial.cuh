// spatial.cuh -- small fixed-size spatial algebra for the device recursions,
// templated on the arithmetic type (double for the plain form, float for the
// spatial recursions of the mixed form). Everything is register-resident.
#pragma once
#include <cuda_runtime.h>

namespace sbg {

template <class R> struct V3 { R x, y, z; };
template <class R> __device__ __forceinline__ V3<R> mk3(R a, R b, R c) { return V3<R>{a, b, c}; }
template <class R> __device__ __forceinline__ V3<R> z3() { return V3<R>{R(0), R(0), R(0)}; }
template <class R> __device__ __forceinline__ V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> __device__ __forceinline__ V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> __device__ __forceinline__ V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> __device__ __forceinline__ V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> __device__ __forceinline__ R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> __device__ __forceinline__ V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// a + s*b
template <class R> __device__ __forceinline__ V3<R> axpy(V3<R> a, R s, V3<R> b) {
    return {a.x + s * b.x, a.y + s * b.y, a.z + s * b.z};
}

// Rotation / general 3x3, row-major.
template <class R> struct M3 { R a[9]; };
template <class R> __device__ __forceinline__ M3<R> ident3() {
    M3<R> m;
#pragma unroll
    for (int i = 0; i < 9; ++i) m.a[i] = R((i % 4) == 0 ? 1 : 0);
    return m;
}
template <class R> __device__ __forceinline__ V3<R> mul(const M3<R>& m, V3<R> v) {
    return {m.a[0] * v.x + m.a[1] * v.y + m.a[2] * v.z,
            m.a[3] * v.x + m.a[4] * v.y + m.a[5] * v.z,
            m.a[6] * v.x + m.a[7] * v.y + m.a[8] * v.z};
}
template <class R> __device__ __forceinline__ V3<R> mulT(const M3<R>& m, V3<R> v) {
    return {m.a[0] * v.x + m.a[3] * v.y + m.a[6] * v.z,
            m.a[1] * v.x + m.a[4] * v.y + m.a[7] * v.z,
            m.a[2] * v.x + m.a[5] * v.y + m.a[8] * v.z};
}
template <class R> __device__ __forceinline__ M3<R> mul(const M3<R>& A, const M3<R>& B) {
    M3<R> C;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            C.a[3 * i + j] = A.a[3 * i] * B.a[j] + A.a[3 * i + 1] * B.a[3 + j] + A.a[3 * i + 2] * B.a[6 + j];
    return C;
}
template <class R> __device__ __forceinline__ V3<R> col(const M3<R>& m, int j) { return {m.a[j], m.a[3 + j], m.a[6 + j]}; }

// Symmetric 3x3: xx yy zz xy xz yz
template <class R> struct S3 { R xx, yy, zz, xy, xz, yz; };
template <class R> __device__ __forceinline__ V3<R> mul(const S3<R>& s, V3<R> v) {
    return {s.xx * v.x + s.xy * v.y + s.xz * v.z,
            s.xy * v.x + s.yy * v.y + s.yz * v.z,
            s.xz * v.x + s.yz * v.y + s.zz * v.z};
}
// R * S * R^T
template <class R> __device__ __forceinline__ S3<R> reexpress(const M3<R>& Rm, const S3<R>& S) {
    // rows of R*S
    V3<R> r0 = mul(S, mk3(Rm.a[0], Rm.a[1], Rm.a[2]));
    V3<R> r1 = mul(S, mk3(Rm.a[3], Rm.a[4], Rm.a[5]));
    V3<R> r2 = mul(S, mk3(Rm.a[6], Rm.a[7], Rm.a[8]));
    const V3<R> c0 = mk3(Rm.a[0], Rm.a[1], Rm.a[2]), c1 = mk3(Rm.a[3], Rm.a[4], Rm.a[5]), c2 = mk3(Rm.a[6], Rm.a[7], Rm.a[8]);
    return S3<R>{dot(r0, c0), dot(r1, c1), dot(r2, c2), dot(r1, c0), dot(r2, c0), dot(r2, c1)};
}

// Articulated body inertia P = [J F; ~F M], M and J symmetric.
template <class R> struct AB { S3<R> M, J; M3<R> F; };

// (J*w + F*v, ~F*w + M*v)
template <class R> __device__ __forceinline__ void abmul(const AB<R>& P, V3<R> w, V3<R> v, V3<R>& ow, V3<R>& ov) {
    ow = mul(P.J, w) + mul(P.F, v);
    ov = mulT(P.F, w) + mul(P.M, v);
}

// P shifted by -s (rigid shift of an articulated inertia toward the parent
// origin): F' = F + s_x*M, J' = J + sym(s_x*~F - F'*s_x).
template <class R> __device__ __forceinline__ AB<R> abshift(const AB<R>& P, V3<R> s) {
    AB<R> o;
    o.M = P.M;
    const R x = s.x, y = s.y, z = s.z;
    const S3<R>& m = P.M;
    // s_x * M
    o.F.a[0] = P.F.a[0] + (y * m.xz - z * m.xy);
    o.F.a[1] = P.F.a[1] + (y * m.yz - z * m.yy);
    o.F.a[2] = P.F.a[2] + (y * m.zz - z * m.yz);
    o.F.a[3] = P.F.a[3] + (z * m.xx - x * m.xz);
    o.F.a[4] = P.F.a[4] + (z * m.xy - x * m.yz);
    o.F.a[5] = P.F.a[5] + (z * m.xz - x * m.zz);
    o.F.a[6] = P.F.a[6] + (x * m.xy - y * m.xx);
    o.F.a[7] = P.F.a[7] + (x * m.yy - y * m.xy);
    o.F.a[8] = P.F.a[8] + (x * m.yz - y * m.xz);
    // lower half of s_x*Ft - G*s_x with Ft = ~F (old), G = F' (new)
    const R* F = P.F.a;   // F(i,j) = F[3i+j]; Ft(i,j) = F[3j+i]
    const R* G = o.F.a;
#define FT(i, j) F[3 * (j) + (i)]
#define GG(i, j) G[3 * (i) + (j)]
    const R h00 = y * (FT(2, 0) + GG(0, 2)) - z * (FT(1, 0) + GG(0, 1));
    const R h10 = z * (FT(0, 0) - GG(1, 1)) - x * FT(2, 0) + y * GG(1, 2);
    const R h11 = z * (FT(0, 1) + GG(1, 0)) - x * (FT(2, 1) + GG(1, 2));
    const R h20 = x * FT(1, 0) - z * GG(2, 1) - y * (FT(0, 0) - GG(2, 2));
    const R h21 = x * (FT(1, 1) - GG(2, 2)) - y * FT(0, 1) + z * GG(2, 0);
    const R h22 = x * (FT(1, 2) + GG(2, 1)) - y * (FT(0, 2) + GG(2, 0));
#undef FT
#undef GG
    o.J.xx = P.J.xx + h00;
    o.J.xy = P.J.xy + h10;
    o.J.yy = P.J.yy + h11;
    o.J.xz = P.J.xz + h20;
    o.J.yz = P.J.yz + h21;
    o.J.zz = P.J.zz + h22;
    return o;
}

}  // namespace sbg
