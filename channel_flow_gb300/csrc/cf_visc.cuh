// Viscous and heat-flux terms (Viscous_terms.cpp:15-886).
//
// Three kernels: (1) primitive u, v, w, T of every cell into scratch (the
// reference repeats this conversion for each of the 13 neighbours with the
// same expression, so precomputing it once changes no value); (2) for every
// cell of i = 3..gend+1, j = 2..nyy, k = 2..nzz the x-, y- and z-face
// fluxes on its low faces into the caller's LL2..5 / ML2..5 / NL2..5 arrays,
// as the reference does; (3) the central divergence vF2..vF5.
#pragma once
#include "cf_common.cuh"


namespace CF_NS {

// the primitive scratch holds the compute type: FP64 (four arrays), or in
// the FP32 build one float4 (u, v, w, T) per cell over the first two
// arrays' allocation, so the face kernels' nine to eleven neighbour reads
// are one 16-byte load each and need no FP64 -> FP32 conversion (a
// conversion issues to GB300's FP64 pipe, 1/64 of the FP32 rate)
__device__ __forceinline__ void prim_st(double *p, size_t q, double v) { p[q] = v; }
__device__ __forceinline__ void prim_st(double *p, size_t q, float v) { reinterpret_cast<float *>(p)[q] = v; }
template <typename T>
__device__ __forceinline__ T prim_ld(const double *p, size_t q);
template <>
__device__ __forceinline__ double prim_ld<double>(const double *p, size_t q) { return p[q]; }
template <>
__device__ __forceinline__ float prim_ld<float>(const double *p, size_t q)
{
    return reinterpret_cast<const float *>(p)[q];
}

template <typename T>
__global__ void k_visc_prim(cf_dims d, cf_visc_args a, size_t n)
{
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const T K = CF_DC(T, d, K), R = CF_DC(T, d, R);
    T rho = T(a.U[0][q]);
#ifdef CF_FAST_MATH
    const T irho = frcp<T>(rho);
    T U = T(a.U[1][q]) * irho;
    T V = T(a.U[2][q]) * irho;
    T W = T(a.U[3][q]) * irho;
#else
    T U = T(a.U[1][q]) / rho;
    T V = T(a.U[2][q]) / rho;
    T W = T(a.U[3][q]) / rho;
#endif
    T VV = U * U + V * V + W * W;
    T Jq = T(a.J[q]);
    T P = (T(a.U[4][q]) - T(0.5) * rho * VV) * (K - T(1)) * Jq;
    T Tt = P / (rho * R) / Jq;
    if (sizeof(T) == 4) {
        reinterpret_cast<float4 *>(a.prim[0])[q] = make_float4(float(U), float(V), float(W), float(Tt));
    } else {
        prim_st(a.prim[0], q, U);
        prim_st(a.prim[1], q, V);
        prim_st(a.prim[2], q, W);
        prim_st(a.prim[3], q, Tt);
    }
}

template <typename T>
struct vgrad {
    T du, dv, dw, du2, dv2, dw2, duv, dvw, duw, dT;
};
template <typename T>
struct vcell {
    T u, v, w, t;
};

template <typename T>
__device__ __forceinline__ vcell<T> ld(const cf_visc_args &a, size_t q)
{
    return vcell<T>{prim_ld<T>(a.prim[0], q), prim_ld<T>(a.prim[1], q), prim_ld<T>(a.prim[2], q),
                    prim_ld<T>(a.prim[3], q)};
}
template <>
__device__ __forceinline__ vcell<float> ld<float>(const cf_visc_args &a, size_t q)
{
    const float4 v = __ldg(reinterpret_cast<const float4 *>(a.prim[0]) + q);
    return vcell<float>{v.x, v.y, v.z, v.w};
}

// one-sided difference c - n (Viscous_terms.cpp:400-415)
template <typename T>
__device__ __forceinline__ vgrad<T> g2(vcell<T> c, vcell<T> n, T inv)
{
    vgrad<T> d;
    d.du = (c.u - n.u) * inv;
    d.dv = (c.v - n.v) * inv;
    d.dw = (c.w - n.w) * inv;
    d.du2 = (c.u * c.u - n.u * n.u) * inv;
    d.dv2 = (c.v * c.v - n.v * n.v) * inv;
    d.dw2 = (c.w * c.w - n.w * n.w) * inv;
    d.duv = (c.u * c.v - n.u * n.v) * inv;
    d.dvw = (c.v * c.w - n.v * n.w) * inv;
    d.duw = (c.u * c.w - n.u * n.w) * inv;
    d.dT = (c.t - n.t) * inv;
    return d;
}
// four-point tangential difference p + q - r - s (Viscous_terms.cpp:419-451);
// the mixed products take their second factor from q2, which reproduces
// the z-face y-derivative kUj*iVj of Viscous_terms.cpp:728-730
template <typename T>
__device__ __forceinline__ vgrad<T> g4(vcell<T> p, vcell<T> q, vcell<T> r, vcell<T> s, vcell<T> q2, T inv)
{
    vgrad<T> d;
    d.du = (p.u + q.u - r.u - s.u) * inv;
    d.dv = (p.v + q.v - r.v - s.v) * inv;
    d.dw = (p.w + q.w - r.w - s.w) * inv;
    d.du2 = (p.u * p.u + q.u * q.u - r.u * r.u - s.u * s.u) * inv;
    d.dv2 = (p.v * p.v + q.v * q.v - r.v * r.v - s.v * s.v) * inv;
    d.dw2 = (p.w * p.w + q.w * q.w - r.w * r.w - s.w * s.w) * inv;
    d.duv = (p.u * p.v + q.u * q2.v - r.u * r.v - s.u * s.v) * inv;
    d.dvw = (p.v * p.w + q.v * q2.w - r.v * r.w - s.v * s.w) * inv;
    d.duw = (p.u * p.w + q.u * q2.w - r.u * r.w - s.u * s.w) * inv;
    d.dT = (p.t + q.t - r.t - s.t) * inv;
    return d;
}

// coefficient sets of one face (Viscous_terms.cpp:471-526)
template <typename T>
struct vsym {
    T s1, s2, s3, s4, s5, s6, s7;
};
template <typename T>
struct vcross {
    T x1, x2, x3, x4, x5, x6, x7, x8, x9, x10;
};
template <typename T>
__device__ __forceinline__ vsym<T> csym(T p0, T p1, T p2)
{
    vsym<T> c;
    c.s1 = (T(4.) / T(3)) * p0 * p0 + p1 * p1 + p2 * p2;
    c.s2 = p0 * p0 + (T(4.) / T(3)) * p1 * p1 + p2 * p2;
    c.s3 = p0 * p0 + p1 * p1 + (T(4.) / T(3)) * p2 * p2;
    c.s4 = p0 * p0 + p1 * p1 + p2 * p2;
    c.s5 = (T(1.) / T(3)) * p0 * p1;
    c.s6 = (T(1.) / T(3)) * p1 * p2;
    c.s7 = (T(1.) / T(3)) * p0 * p2;
    return c;
}
template <typename T>
__device__ __forceinline__ vcross<T> ccross(T p0, T p1, T p2, T q0, T q1, T q2)
{
    vcross<T> c;
    c.x1 = (T(4.) / T(3)) * p0 * q0 + p1 * q1 + p2 * q2;
    c.x2 = p0 * q0 + (T(4.) / T(3)) * p1 * q1 + p2 * q2;
    c.x3 = p0 * q0 + p1 * q1 + (T(4.) / T(3)) * p2 * q2;
    c.x4 = p0 * q0 + p1 * q1 + p2 * q2;
    c.x5 = p0 * q1 - (T(2.) / T(3)) * p1 * q0;
    c.x6 = p0 * q2 - (T(2.) / T(3)) * p2 * q0;
    c.x7 = p1 * q0 - (T(2.) / T(3)) * p0 * q1;
    c.x8 = p1 * q2 - (T(2.) / T(3)) * p2 * q1;
    c.x9 = p2 * q0 - (T(2.) / T(3)) * p0 * q2;
    c.x10 = p2 * q1 - (T(2.) / T(3)) * p1 * q2;
    return c;
}

// grid constants of the face fluxes
template <typename T>
struct vconst {
    T K, Cv, mu_E, Pr_E, iPr, invXI, invET, invZT, inv4XI, inv4ET, inv4ZT;
};
template <typename T>
__device__ __forceinline__ vconst<T> visc_consts(const cf_dims &d)
{
    vconst<T> k;
    k.K = CF_DC(T, d, K);
    k.Cv = CF_DC(T, d, Cv);
    k.mu_E = CF_DC(T, d, mu_L);
    k.Pr_E = CF_DC(T, d, Pr_L);
#ifdef CF_FAST_MATH
    k.iPr = CF_DINV(T, d, Pr_L, iPr);
#else
    k.iPr = T(0);
#endif
    k.invXI = CF_DINV(T, d, dXI, idXI);
    k.invET = CF_DINV(T, d, dET, idET);
    k.invZT = CF_DINV(T, d, dZT, idZT);
#ifdef CF_FAST_MATH
    // 1/(4 d) = (1/d)/4 exactly: a power-of-two scaling commutes with rounding
    k.inv4XI = T(0.25) * k.invXI;
    k.inv4ET = T(0.25) * k.invET;
    k.inv4ZT = T(0.25) * k.invZT;
#else
    k.inv4XI = T(1.) / (T(4) * CF_DC(T, d, dXI));
    k.inv4ET = T(1.) / (T(4) * CF_DC(T, d, dET));
    k.inv4ZT = T(1.) / (T(4) * CF_DC(T, d, dZT));
#endif
    return k;
}

// the face's J and nine metrics
template <typename T>
struct vmet {
    T Jf, m[9];
};
template <typename T>
__device__ __forceinline__ vmet<T> visc_met(const cf_visc_args &a, int face, size_t f)
{
    vmet<T> r;
    r.Jf = met_ld<T>(a.Jf[face], a.Jf32[face], f);
#pragma unroll
    for (int n = 0; n < 9; n++) r.m[n] = met_ld<T>(a.mf[face][n], a.mf32[face][n], f);
    return r;
}

#ifdef CF_FAST_MATH
// the contracted and FP32 builds multiply by reciprocals of Pr and J_f
#define CF_VPR(x) ((x) * k.iPr)
#define CF_VJF(x) ((x) * iJf)
#else
#define CF_VPR(x) ((x) / (k.Pr_E))
#define CF_VJF(x) ((x) / M.Jf)
#endif

// x face between cells i-1 and i (Viscous_terms.cpp:398-547): c = (i,j,k),
// im = (i-1,j,k), the tangential neighbours of both planes; out = LL2..5
template <typename T>
__device__ __forceinline__ void visc_face_x(const vconst<T> &k, const vmet<T> &M, vcell<T> c, vcell<T> im,
                                            vcell<T> jp, vcell<T> jm, vcell<T> imjp, vcell<T> imjm, vcell<T> kp,
                                            vcell<T> km, vcell<T> imkp, vcell<T> imkm, T *out)
{
    const T K = k.K, Cv = k.Cv, mu_E = k.mu_E;
    vgrad<T> X = g2<T>(c, im, k.invXI);
    vgrad<T> Y = g4<T>(jp, imjp, jm, imjm, imjp, k.inv4ET);
    vgrad<T> Z = g4<T>(kp, imkp, km, imkm, imkp, k.inv4ZT);
    const T m0 = M.m[0], m1 = M.m[1], m2 = M.m[2];
    vsym<T> A = csym<T>(m0, m1, m2);
    vcross<T> D = ccross<T>(m0, m1, m2, M.m[3], M.m[4], M.m[5]);
    vcross<T> E = ccross<T>(m0, m1, m2, M.m[6], M.m[7], M.m[8]);
    T Ux = T(0.5) * (c.u + im.u), Vx = T(0.5) * (c.v + im.v), Wx = T(0.5) * (c.w + im.w);
#ifdef CF_FAST_MATH
    const T iJf = frcp<T>(M.Jf);
#endif
    out[0] = T(CF_VJF(mu_E * (A.s1 * X.du + A.s5 * X.dv + A.s7 * X.dw + D.x1 * Y.du + D.x7 * Y.dv + D.x9 * Y.dw + E.x1 * Z.du + E.x7 * Z.dv + E.x9 * Z.dw)));
    out[1] = T(CF_VJF(mu_E * (A.s5 * X.du + A.s2 * X.dv + A.s6 * X.dw + D.x5 * Y.du + D.x2 * Y.dv + D.x10 * Y.dw + E.x5 * Z.du + E.x2 * Z.dv + E.x10 * Z.dw)));
    out[2] = T(CF_VJF(mu_E * (A.s7 * X.du + A.s6 * X.dv + A.s3 * X.dw + D.x6 * Y.du + D.x8 * Y.dv + D.x3 * Y.dw + E.x6 * Z.du + E.x8 * Z.dv + E.x3 * Z.dw)));
    out[3] = T(CF_VJF(mu_E * (T(0.5) * A.s1 * X.du2 + T(0.5) * A.s2 * X.dv2 + T(0.5) * A.s3 * X.dw2 + A.s5 * X.duv + A.s6 * X.dvw + A.s7 * X.duw + CF_VPR(Cv * K * A.s4 * X.dT) +
        T(0.5) * D.x1 * Y.du2 + T(0.5) * D.x2 * Y.dv2 + T(0.5) * D.x3 * Y.dw2 + D.x5 * Vx * Y.du + D.x6 * Wx * Y.du + D.x7 * Ux * Y.dv + D.x8 * Wx * Y.dv + D.x9 * Ux * Y.dw + D.x10 * Vx * Y.dw + CF_VPR(Cv * K * D.x4 * Y.dT) +
        T(0.5) * E.x1 * Z.du2 + T(0.5) * E.x2 * Z.dv2 + T(0.5) * E.x3 * Z.dw2 + E.x5 * Vx * Z.du + E.x6 * Wx * Z.du + E.x7 * Ux * Z.dv + E.x8 * Wx * Z.dv + E.x9 * Ux * Z.dw + E.x10 * Vx * Z.dw + CF_VPR(Cv * K * E.x4 * Z.dT))));
}

// y face between j-1 and j (Viscous_terms.cpp:550-695); out = ML2..5
template <typename T>
__device__ __forceinline__ void visc_face_y(const vconst<T> &k, const vmet<T> &M, vcell<T> c, vcell<T> jm,
                                            vcell<T> ip, vcell<T> im, vcell<T> ipjm, vcell<T> imjm, vcell<T> kp,
                                            vcell<T> km, vcell<T> jmkp, vcell<T> jmkm, T *out)
{
    const T K = k.K, Cv = k.Cv, mu_E = k.mu_E;
    vgrad<T> X = g4<T>(ip, ipjm, im, imjm, ipjm, k.inv4XI);
    vgrad<T> Y = g2<T>(c, jm, k.invET);
    vgrad<T> Z = g4<T>(kp, jmkp, km, jmkm, jmkp, k.inv4ZT);
    const T m0 = M.m[0], m1 = M.m[1], m2 = M.m[2];
    const T e0 = M.m[3], e1 = M.m[4], e2 = M.m[5];
    vsym<T> B = csym<T>(e0, e1, e2);
    vcross<T> D = ccross<T>(m0, m1, m2, e0, e1, e2);
    vcross<T> F = ccross<T>(e0, e1, e2, M.m[6], M.m[7], M.m[8]);
    T Uy = T(0.5) * (c.u + jm.u), Vy = T(0.5) * (c.v + jm.v), Wy = T(0.5) * (c.w + jm.w);
#ifdef CF_FAST_MATH
    const T iJf = frcp<T>(M.Jf);
#endif
    out[0] = T(CF_VJF(mu_E * (D.x1 * X.du + D.x5 * X.dv + D.x6 * X.dw + B.s1 * Y.du + B.s5 * Y.dv + B.s7 * Y.dw + F.x1 * Z.du + F.x7 * Z.dv + F.x9 * Z.dw)));
    out[1] = T(CF_VJF(mu_E * (D.x7 * X.du + D.x2 * X.dv + D.x8 * X.dw + B.s5 * Y.du + B.s2 * Y.dv + B.s6 * Y.dw + F.x5 * Z.du + F.x2 * Z.dv + F.x10 * Z.dw)));
    out[2] = T(CF_VJF(mu_E * (D.x9 * X.du + D.x10 * X.dv + D.x3 * X.dw + B.s7 * Y.du + B.s6 * Y.dv + B.s3 * Y.dw + F.x6 * Z.du + F.x8 * Z.dv + F.x3 * Z.dw)));
    out[3] = T(CF_VJF(mu_E * (T(0.5) * B.s1 * Y.du2 + T(0.5) * B.s2 * Y.dv2 + T(0.5) * B.s3 * Y.dw2 + B.s5 * Y.duv + B.s6 * Y.dvw + B.s7 * Y.duw + CF_VPR(Cv * K * B.s4 * Y.dT) +
        T(0.5) * D.x1 * X.du2 + T(0.5) * D.x2 * X.dv2 + T(0.5) * D.x3 * X.dw2 + D.x5 * Uy * X.dv + D.x6 * Uy * X.dw + D.x7 * Vy * X.du + D.x8 * Vy * X.dw + D.x9 * Wy * X.du + D.x10 * Wy * X.dv + CF_VPR(Cv * K * D.x4 * X.dT) +
        T(0.5) * F.x1 * Z.du2 + T(0.5) * F.x2 * Z.dv2 + T(0.5) * F.x3 * Z.dw2 + F.x5 * Vy * Z.du + F.x6 * Wy * Z.du + F.x7 * Uy * Z.dv + F.x8 * Wy * Z.dv + F.x9 * Uy * Z.dw + F.x10 * Vy * Z.dw + CF_VPR(Cv * K * F.x4 * Z.dT))));
}

// z face between k-1 and k (Viscous_terms.cpp:698-841); out = NL2..5
template <typename T>
__device__ __forceinline__ void visc_face_z(const vconst<T> &k, const vmet<T> &M, vcell<T> c, vcell<T> km,
                                            vcell<T> ip, vcell<T> im, vcell<T> ipkm, vcell<T> imkm, vcell<T> jp,
                                            vcell<T> jm, vcell<T> jpkm, vcell<T> jmkm, vcell<T> imjp, T *out)
{
    const T K = k.K, Cv = k.Cv, mu_E = k.mu_E;
    vgrad<T> X = g4<T>(ip, ipkm, im, imkm, ipkm, k.inv4XI);
    vgrad<T> Y = g4<T>(jp, jpkm, jm, jmkm, imjp, k.inv4ET);
    vgrad<T> Z = g2<T>(c, km, k.invZT);
    const T z0 = M.m[6], z1 = M.m[7], z2 = M.m[8];
    vsym<T> Cc = csym<T>(z0, z1, z2);
    vcross<T> E = ccross<T>(M.m[0], M.m[1], M.m[2], z0, z1, z2);
    vcross<T> F = ccross<T>(M.m[3], M.m[4], M.m[5], z0, z1, z2);
    T Uz = T(0.5) * (c.u + km.u), Vz = T(0.5) * (c.v + km.v), Wz = T(0.5) * (c.w + km.w);
#ifdef CF_FAST_MATH
    const T iJf = frcp<T>(M.Jf);
#endif
    out[0] = T(CF_VJF(mu_E * (E.x1 * X.du + E.x5 * X.dv + E.x6 * X.dw + F.x1 * Y.du + F.x5 * Y.dv + F.x6 * Y.dw + Cc.s1 * Z.du + Cc.s5 * Z.dv + Cc.s7 * Z.dw)));
    out[1] = T(CF_VJF(mu_E * (E.x7 * X.du + E.x2 * X.dv + E.x8 * X.dw + F.x7 * Y.du + F.x2 * Y.dv + F.x8 * Y.dw + Cc.s5 * Z.du + Cc.s2 * Z.dv + Cc.s6 * Z.dw)));
    out[2] = T(CF_VJF(mu_E * (E.x9 * X.du + E.x10 * X.dv + E.x3 * X.dw + F.x9 * Y.du + F.x10 * Y.dv + F.x3 * Y.dw + Cc.s7 * Z.du + Cc.s6 * Z.dv + Cc.s3 * Z.dw)));
    out[3] = T(CF_VJF(mu_E * (T(0.5) * Cc.s1 * Z.du2 + T(0.5) * Cc.s2 * Z.dv2 + T(0.5) * Cc.s3 * Z.dw2 + Cc.s5 * Z.duv + Cc.s6 * Z.dvw + Cc.s7 * Z.duw + CF_VPR(Cv * K * Cc.s4 * Z.dT) +
        T(0.5) * E.x1 * X.du2 + T(0.5) * E.x2 * X.dv2 + T(0.5) * E.x3 * X.dw2 + E.x5 * Uz * X.dv + E.x6 * Uz * X.dw + E.x7 * Vz * X.du + E.x8 * Vz * X.dw + E.x9 * Wz * X.du + E.x10 * Wz * X.dv + CF_VPR(Cv * K * E.x4 * X.dT) +
        T(0.5) * F.x1 * Y.du2 + T(0.5) * F.x2 * Y.dv2 + T(0.5) * F.x3 * Y.dw2 + F.x5 * Uz * Y.dv + F.x6 * Uz * Y.dw + F.x7 * Vz * Y.du + F.x8 * Vz * Y.dw + F.x9 * Wz * Y.du + F.x10 * Wz * Y.dv + CF_VPR(Cv * K * F.x4 * Y.dT))));
}

// FACE 0/1/2: the x, y or z face of every cell, one launch each (the
// register footprint of one face: in FP32 twice the resident warps of a
// kernel doing all three faces, which measured slower).  Blocks per SM:
// FP32 3; FP64 2 in the contracted build (128 registers, no spills), 1 in
// the no-FMA build (whose longer expression trees would spill at 128)
#ifdef CF_FAST_MATH
constexpr int VF_FP64_BLOCKS = 2;
#else
constexpr int VF_FP64_BLOCKS = 1;
#endif
template <typename T, int FACE>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : VF_FP64_BLOCKS) k_visc_faces(cf_dims d, cf_visc_args a, cf_box b)
{
    CF_BOX_INDEX(b, i, j, k);
    const vconst<T> kc = visc_consts<T>(d);
    const size_t q = d.ix(i, j, k), f = d.ix(i - 1, j - 1, k - 1);
    const vcell<T> c = ld<T>(a, q);
    const vcell<T> im = ld<T>(a, d.ix(i - 1, j, k)), jm = ld<T>(a, d.ix(i, j - 1, k)),
                   km = ld<T>(a, d.ix(i, j, k - 1));
    const vcell<T> ip = FACE != 0 ? ld<T>(a, d.ix(i + 1, j, k)) : c;
    const vcell<T> jp = FACE != 1 ? ld<T>(a, d.ix(i, j + 1, k)) : c;
    const vcell<T> kp = FACE != 2 ? ld<T>(a, d.ix(i, j, k + 1)) : c;
    const vmet<T> M = visc_met<T>(a, FACE, f);
    T out[4];
    if (FACE == 0) {
        const vcell<T> imjp = ld<T>(a, d.ix(i - 1, j + 1, k)), imkp = ld<T>(a, d.ix(i - 1, j, k + 1));
        const vcell<T> imjm = ld<T>(a, d.ix(i - 1, j - 1, k)), imkm = ld<T>(a, d.ix(i - 1, j, k - 1));
        visc_face_x<T>(kc, M, c, im, jp, jm, imjp, imjm, kp, km, imkp, imkm, out);
#pragma unroll
        for (int v = 0; v < 4; v++) rhs_put<T>(a.LL[v], q, out[v], a.f32_io);
    }
    if (FACE == 1) {
        const vcell<T> ipjm = ld<T>(a, d.ix(i + 1, j - 1, k)), imjm = ld<T>(a, d.ix(i - 1, j - 1, k));
        const vcell<T> jmkp = ld<T>(a, d.ix(i, j - 1, k + 1)), jmkm = ld<T>(a, d.ix(i, j - 1, k - 1));
        visc_face_y<T>(kc, M, c, jm, ip, im, ipjm, imjm, kp, km, jmkp, jmkm, out);
#pragma unroll
        for (int v = 0; v < 4; v++) rhs_put<T>(a.ML[v], q, out[v], a.f32_io);
    }
    if (FACE == 2) {
        const vcell<T> ipkm = ld<T>(a, d.ix(i + 1, j, k - 1)), imkm = ld<T>(a, d.ix(i - 1, j, k - 1));
        const vcell<T> jpkm = ld<T>(a, d.ix(i, j + 1, k - 1)), jmkm = ld<T>(a, d.ix(i, j - 1, k - 1));
        const vcell<T> imjp = ld<T>(a, d.ix(i - 1, j + 1, k));
        visc_face_z<T>(kc, M, c, km, ip, im, ipkm, imkm, jp, jm, jpkm, jmkm, imjp, out);
#pragma unroll
        for (int v = 0; v < 4; v++) rhs_put<T>(a.NL[v], q, out[v], a.f32_io);
    }
}

#undef CF_VPR
#undef CF_VJF

// The FP32 step driver's viscous terms in one pass (its face fluxes are
// read by nothing else).  A block owns VM_TJ x VM_TK = 8 x 32 (j, k)
// columns of cells and marches through a chunk of x planes.  The primitives
// of three planes (i-1, i, i+1) with a one-cell halo in j and k sit in
// shared memory as float4, formed from the sub-iteration's FP32 copies of
// U_ and J with k_visc_prim's arithmetic.  At plane i the block forms the x
// face between i and i+1 of each of its cells (the face between i-1 and i
// is the previous plane's, kept in registers), the y faces of rows j0 ..
// j0+8 and the z faces of columns k0 .. k0+32 of plane i, and the
// divergence vF of its cells, each with the arithmetic of k_visc_faces and
// k_visc_div, so the results equal the five-kernel form's.
constexpr int VM_TJ = 8, VM_TK = 32, VM_HJ = VM_TJ + 2, VM_HK = VM_TK + 2;

__device__ __forceinline__ float4 visc_prim32(const cf_dims &d, const cf_visc_args &a, size_t q)
{
    const float K = d.f_K, R = d.f_R;
    const float rho = a.U32[0][q];
#ifdef CF_FAST_MATH
    const float irho = frcp<float>(rho);
    const float U = a.U32[1][q] * irho, V = a.U32[2][q] * irho, W = a.U32[3][q] * irho;
#else
    const float U = a.U32[1][q] / rho, V = a.U32[2][q] / rho, W = a.U32[3][q] / rho;
#endif
    const float VV = U * U + V * V + W * W;
    const float Jq = a.J32[q];
    const float P = (a.U32[4][q] - 0.5f * rho * VV) * (K - 1.0f) * Jq;
    const float Tt = P / (rho * R) / Jq;
    return make_float4(U, V, W, Tt);
}

__global__ void __launch_bounds__(256, 3) k_visc_march(cf_dims d, cf_visc_args a, int fti)
{
    __shared__ float4 sp[3][VM_HJ][VM_HK];
    __shared__ float syf[4][VM_TJ + 1][VM_TK];
    __shared__ float szf[4][VM_TJ][VM_TK + 1];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
    const int k0 = 2 + (int)blockIdx.x * VM_TK, j0 = 2 + (int)blockIdx.y * VM_TJ;
    const int i0 = 3 + (int)blockIdx.z * fti, i1 = min(i0 + fti - 1, d.gend);
    const vconst<float> kc = visc_consts<float>(d);
    const int j = j0 + ty, k = k0 + tx;
    const bool cell_ok = j <= d.ny && k <= d.nz;
    auto load_plane = [&](int ii) {
        float4(*dst)[VM_HK] = sp[ii % 3];
        for (int e = tid; e < VM_HJ * VM_HK; e += 256) {
            const int r = e / VM_HK, c = e % VM_HK;
            const int jj = j0 - 1 + r, kk = k0 - 1 + c;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (jj <= d.ny + 2 && kk <= d.nz + 2) v = visc_prim32(d, a, d.ix(ii, jj, kk));
            dst[r][c] = v;
        }
    };
    // the primitives of cell (ii, jj, kk) of the block's halo
    auto P = [&](int ii, int jj, int kk) -> vcell<float> {
        const float4 v = sp[ii % 3][jj - j0 + 1][kk - k0 + 1];
        return vcell<float>{v.x, v.y, v.z, v.w};
    };
    auto xface = [&](int I, float *out) {
        const vmet<float> M = visc_met<float>(a, 0, d.ix(I - 1, j - 1, k - 1));
        visc_face_x<float>(kc, M, P(I, j, k), P(I - 1, j, k), P(I, j + 1, k), P(I, j - 1, k), P(I - 1, j + 1, k),
                           P(I - 1, j - 1, k), P(I, j, k + 1), P(I, j, k - 1), P(I - 1, j, k + 1),
                           P(I - 1, j, k - 1), out);
    };
    auto yface = [&](int I, int row) {
        const int jj = j0 + row;
        float out[4];
        const vmet<float> M = visc_met<float>(a, 1, d.ix(I - 1, jj - 1, k - 1));
        visc_face_y<float>(kc, M, P(I, jj, k), P(I, jj - 1, k), P(I + 1, jj, k), P(I - 1, jj, k),
                           P(I + 1, jj - 1, k), P(I - 1, jj - 1, k), P(I, jj, k + 1), P(I, jj, k - 1),
                           P(I, jj - 1, k + 1), P(I, jj - 1, k - 1), out);
#pragma unroll
        for (int v = 0; v < 4; v++) syf[v][row][tx] = out[v];
    };
    auto zface = [&](int I, int col) {
        const int kk = k0 + col;
        float out[4];
        const vmet<float> M = visc_met<float>(a, 2, d.ix(I - 1, j - 1, kk - 1));
        visc_face_z<float>(kc, M, P(I, j, kk), P(I, j, kk - 1), P(I + 1, j, kk), P(I - 1, j, kk),
                           P(I + 1, j, kk - 1), P(I - 1, j, kk - 1), P(I, j + 1, kk), P(I, j - 1, kk),
                           P(I, j + 1, kk - 1), P(I, j - 1, kk - 1), P(I - 1, j + 1, kk), out);
#pragma unroll
        for (int v = 0; v < 4; v++) szf[v][ty][col] = out[v];
    };
    load_plane(i0 - 1);
    load_plane(i0);
    __syncthreads();
    float xlo[4] = {0.f, 0.f, 0.f, 0.f};
    if (cell_ok) xface(i0, xlo);
    for (int i = i0; i <= i1; i++) {
        load_plane(i + 1);
        __syncthreads();
        float xhi[4] = {0.f, 0.f, 0.f, 0.f};
        if (cell_ok) xface(i + 1, xhi);
        // y faces of rows j0 + ty (row 8 by the first row of threads), z
        // faces of columns k0 + tx (column 32 by the first column)
        if (j <= d.ny + 1 && k <= d.nz) yface(i, ty);
        if (ty == 0 && j0 + VM_TJ <= d.ny + 1 && k <= d.nz) yface(i, VM_TJ);
        if (j <= d.ny && k <= d.nz + 1) zface(i, tx);
        if (tx == 0 && j <= d.ny && k0 + VM_TK <= d.nz + 1) zface(i, VM_TK);
        __syncthreads();
        if (cell_ok) {
            const size_t q = d.ix(i, j, k);
#pragma unroll
            for (int v = 0; v < 4; v++)
                rhs_put<float>(a.vF[v], q,
                               (xhi[v] - xlo[v]) * kc.invXI + (syf[v][ty + 1][tx] - syf[v][ty][tx]) * kc.invET +
                                   (szf[v][ty][tx + 1] - szf[v][ty][tx]) * kc.invZT,
                               a.f32_io);
        }
#pragma unroll
        for (int v = 0; v < 4; v++) xlo[v] = xhi[v];
    }
}

// Viscous_terms.cpp:854-883
template <typename T>
__global__ void k_visc_div(cf_dims d, cf_visc_args a, cf_box b)
{
    CF_BOX_INDEX(b, i, j, k);
    const T invXI = CF_DINV(T, d, dXI, idXI), invET = CF_DINV(T, d, dET, idET), invZT = CF_DINV(T, d, dZT, idZT);
    const size_t q = d.ix(i, j, k), qi = d.ix(i + 1, j, k), qj = d.ix(i, j + 1, k), qk = q + 1;
#pragma unroll
    for (int v = 0; v < 4; v++) {
        const int f = a.f32_io;
        rhs_put<T>(a.vF[v], q,
                   (rhs_get<T>(a.LL[v], qi, f) - rhs_get<T>(a.LL[v], q, f)) * invXI +
                       (rhs_get<T>(a.ML[v], qj, f) - rhs_get<T>(a.ML[v], q, f)) * invET +
                       (rhs_get<T>(a.NL[v], qk, f) - rhs_get<T>(a.NL[v], q, f)) * invZT, f);
    }
}

template <typename T>
cudaError_t launch_viscous(const cf_dims &d, const cf_visc_args &a, cudaStream_t s)
{
    if (sizeof(T) == 4 && a.f32_io && a.U32[0] && a.J32) {
        // the step driver: one marching pass, x cut into chunks so that the
        // grid holds about four waves of two resident blocks per SM
        static int sms = 0;
        if (!sms) {
            int dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (sms <= 0) sms = 132;
        }
        const int tk = (d.Z_out + VM_TK - 1) / VM_TK, tj = (d.Y_out + VM_TJ - 1) / VM_TJ;
        const int chunks = std::max(1, std::min(d.X_out / 8, (8 * sms + tk * tj - 1) / (tk * tj)));
        const int fti = (d.X_out + chunks - 1) / chunks;
        const dim3 g((unsigned)tk, (unsigned)tj, (unsigned)((d.X_out + fti - 1) / fti));
        k_visc_march<<<g, dim3(32, VM_TJ), 0, s>>>(d, a, fti);
        return cudaGetLastError();
    }
    const size_t n = d.total();
    k_visc_prim<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d, a, n);
    cf_box bf = make_box(3, d.gend + 1, 2, d.ny + 1, 2, d.nz + 1);
    k_visc_faces<T, 0><<<box_grid(bf), box_block(), 0, s>>>(d, a, bf);
    k_visc_faces<T, 1><<<box_grid(bf), box_block(), 0, s>>>(d, a, bf);
    k_visc_faces<T, 2><<<box_grid(bf), box_block(), 0, s>>>(d, a, bf);
    cf_box bd = make_box(3, d.gend, 2, d.ny, 2, d.nz);
    k_visc_div<T><<<box_grid(bd), box_block(), 0, s>>>(d, a, bd);
    return cudaGetLastError();
}

}  // namespace CF_NS
