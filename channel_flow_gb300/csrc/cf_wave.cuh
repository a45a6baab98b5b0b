// Hyperplane LU-SGS sweeps as one persistent wavefront launch per sweep
// (Dual_time_stepping.cpp:563-1250).
//
// The interior is cut into tiles of 4 x 8 x 8 cells (i, j, k).  Cell
// (i,j,k) of the forward sweep needs N of (i-1,j,k), (i,j-1,k), (i,j,k-1)
// only, so a tile can run once its three lower neighbour tiles are done,
// and inside a tile the cells of one local plane li+lj+lk = l are
// independent.  Every cell still sees exactly the inputs of the reference's
// plane-ordered loop, so the results are the same bits; only the order in
// which independent cells are computed changes.
//
// Each cell's contribution to a neighbour, e.g. (-p11 a0 - p12 a1 - p13 a2
// - p14 a3)/dXI of the x split of cell i-1, is a function of that
// neighbour's own split and N alone.  The producing cell therefore forms
// the three terms it owes its upper (forward) or lower (backward)
// neighbours right after its own N, and the consumer adds the three terms
// in the reference's order x + y + z.  Terms stay in shared memory inside a
// tile and cross tile faces through exchange fields in HBM; terms from
// ghost cells (N = 0) are formed by k_lu_tile_pack.
//
// Scheduling: four warps per block; a block claims tiles in topological order
// (atomic counter over a plane-sorted tile list), stages the tile's
// coefficient pack into shared memory with one bulk async copy
// (cp.async.bulk, mbarrier completion) while it waits for the neighbour
// tiles' done flags (acquire loads), runs the tile's local planes, and
// publishes its flag (release).  A block only waits on tiles claimed before
// its own, so the launch cannot deadlock whatever the number of resident
// blocks.  Every wait is bounded; a wait that runs out sets an error word
// the host reads, and the tile proceeds so that no other wait can hang.
#pragma once
#include "cf_lusgs.cuh"

namespace CF_NS {

constexpr int WV_TI = 4, WV_TJ = 8, WV_TK = 8, WV_CELLS = WV_TI * WV_TJ * WV_TK;
constexpr int WV_PACK = 50;          // values per cell of a tile pack
constexpr int WV_STAGE = 44;         // values per cell a sweep stages (forward: 6..49, backward: 0..38)
constexpr int WV_FWD0 = 6;           // first value of the forward window
constexpr unsigned WV_SPIN_LIMIT = CF_WAVE_SPIN_LIMIT;   // polls before a copy wait gives up

// One pack per tile (tile-major; inside a tile value-major, value m of cell
// c = (li*8 + lj)*8 + lk at [m][c]), ordered so that each sweep stages one
// contiguous window of it:
//   0..5    m11 m22 of the x, y, z splits            (backward only)
//   6..35   p12 p13 p14 p21 p31 p41 p51 p52 p53 p54 of x, y, z   (both)
//   36..38  d11 d22 d51                               (both)
//   39..44  p11 p22 of the x, y, z splits             (forward only)
//   45..49  MR1..MR5                                  (forward only)
// The forward sweep stages values 6..49, the backward sweep values 0..38
// (and the forward N of the tile, from cf_wave_args::nl), so the pack is
// written once for both sweeps.
// (cf_wave_args in cf_types.h holds the tiling and the scratch.)
using wave_args = cf_wave_args;
static_assert(WV_TI == CF_WAVE_TI && WV_TJ == CF_WAVE_TJ && WV_TK == CF_WAVE_TK && WV_PACK == CF_WAVE_PACK,
              "tile geometry");

__device__ __forceinline__ void wave_tile_coords(const wave_args &w, int t, int &a, int &b, int &c)
{
    c = t % w.ntk;
    b = (t / w.ntk) % w.ntj;
    a = t / (w.ntk * w.ntj);
}

// the t-th cell of local plane l of a ti x tj x tk tile (li-major order)
__device__ __forceinline__ bool wave_cell(int l, int t, int ti, int tj, int tk, int &li, int &lj, int &lk)
{
    const int lo = max(0, l - (tj - 1) - (tk - 1)), hi = min(ti - 1, l);
    for (int a = lo; a <= hi; a++) {
        const int rem = l - a;
        const int jl = max(0, rem - (tk - 1)), jh = min(tj - 1, rem);
        const int cnt = jh - jl + 1;
        if (cnt <= 0) continue;
        if (t < cnt) {
            li = a;
            lj = jl + t;
            lk = rem - lj;
            return true;
        }
        t -= cnt;
    }
    return false;
}

// The five terms a cell owes a neighbour along one direction (the lower
// form, Dual_time_stepping.cpp:751-811, and the upper form, 1116-1177)
// from its 12 split coefficients P and its N.  The no-FMA build keeps the
// reference's (sum) / dXI; the contracted and FP32 builds store P already
// multiplied by 1/dXI (wave_scale) and skip the division.
template <typename T>
__device__ __forceinline__ T wave_div(T x, const lu_den<T> &den)
{
#ifdef CF_FAST_MATH
    (void)den;
    return x;
#else
    return x / den.den;
#endif
}

template <typename T>
__device__ __forceinline__ void wave_scale(T *P, const lu_den<T> &den)
{
#ifdef CF_FAST_MATH
#pragma unroll
    for (int m = 0; m < 12; m++) P[m] = P[m] * den.rden;
#else
    (void)P;
    (void)den;
#endif
}

template <typename T>
__device__ __forceinline__ void wave_lower_terms(const T *P, const T *a, const lu_den<T> &den, T *o)
{
    // P: p11 p22 p12 p13 p14 p21 p31 p41 p51 p52 p53 p54
    const T p11 = P[0], p22 = P[1], p12 = P[2], p13 = P[3], p14 = P[4], p21 = P[5], p31 = P[6], p41 = P[7],
            p51 = P[8], p52 = P[9], p53 = P[10], p54 = P[11];
    o[0] = wave_div(-p11 * a[0] - p12 * a[1] - p13 * a[2] - p14 * a[3], den);
    o[1] = wave_div(-p21 * a[0] - p22 * a[1], den);
    o[2] = wave_div(-p31 * a[0] - p22 * a[2], den);
    o[3] = wave_div(-p41 * a[0] - p22 * a[3], den);
    o[4] = wave_div(-p51 * a[0] - p52 * a[1] - p53 * a[2] - p54 * a[3] - p22 * a[4], den);
}

template <typename T>
__device__ __forceinline__ void wave_upper_terms(const T *P, const T *a, const lu_den<T> &den, T *o)
{
    // P: m11 m22 p12 p13 p14 p21 p31 p41 p51 p52 p53 p54
    const T m11 = P[0], m22 = P[1], p12 = P[2], p13 = P[3], p14 = P[4], p21 = P[5], p31 = P[6], p41 = P[7],
            p51 = P[8], p52 = P[9], p53 = P[10], p54 = P[11];
    o[0] = wave_div(+m11 * a[0] + p12 * a[1] + p13 * a[2] + p14 * a[3], den);
    o[1] = wave_div(+p21 * a[0] + m22 * a[1], den);
    o[2] = wave_div(+p31 * a[0] + m22 * a[2], den);
    o[3] = wave_div(+p41 * a[0] + m22 * a[3], den);
    o[4] = wave_div(+p51 * a[0] + p52 * a[1] + p53 * a[2] + p54 * a[3] + m22 * a[4], den);
}

template <typename T, bool UPPER>
__device__ __forceinline__ void wave_split12(const lsplit<T> &A, T *o)
{
    o[0] = UPPER ? A.m11 : A.p11;
    o[1] = UPPER ? A.m22 : A.p22;
    o[2] = A.p12; o[3] = A.p13; o[4] = A.p14; o[5] = A.p21;
    o[6] = A.p31; o[7] = A.p41; o[8] = A.p51; o[9] = A.p52; o[10] = A.p53; o[11] = A.p54;
}

// split of direction dir of cell q (state s)
template <typename T>
__device__ __forceinline__ lsplit<T> wave_split(const cf_dims &d, const cf_lu_args &a, size_t q, const lstate<T> &s,
                                                int dir)
{
    return lu_split<T>(s, met_ld<T>(a.m[3 * dir], a.m32[3 * dir], q), met_ld<T>(a.m[3 * dir + 1], a.m32[3 * dir + 1], q), met_ld<T>(a.m[3 * dir + 2], a.m32[3 * dir + 2], q), dir == 0, CF_DC(T, d, K));
}

// face slots: x face cell (lj, lk) -> lj*8 + lk, y face (li, lk) -> li*8 + lk,
// z face (li, lj) -> li*8 + lj; per tile [5][slots]
constexpr int WV_FX = WV_TJ * WV_TK, WV_FY = WV_TI * WV_TK, WV_FZ = WV_TI * WV_TJ;

template <typename T>
__device__ __forceinline__ T *wave_face(const wave_args &w, int dir, int tile)
{
    if (dir == 0) return static_cast<T *>(w.inx) + (size_t)tile * 5 * WV_FX;
    if (dir == 1) return static_cast<T *>(w.iny) + (size_t)tile * 5 * WV_FY;
    return static_cast<T *>(w.inz) + (size_t)tile * 5 * WV_FZ;
}

// terms of ghost cell qg (N = 0) into face slot f of a tile
template <typename T, bool UPPER>
__device__ __forceinline__ void wave_ghost_term(const cf_dims &d, const cf_lu_args &a, size_t qg, int dir,
                                                const lu_den<T> &den, T *face, int nslot, int f)
{
    const lstate<T> s = lu_state<T>(d, a, qg);
    const lsplit<T> A = wave_split<T>(d, a, qg, s, dir);
    T P[12], o[5];
    wave_split12<T, UPPER>(A, P);
    wave_scale<T>(P, den);
    const T zero[5] = {T(0), T(0), T(0), T(0), T(0)};
    if (UPPER) wave_upper_terms<T>(P, zero, den, o);
    else wave_lower_terms<T>(P, zero, den, o);
#pragma unroll
    for (int n = 0; n < 5; n++) face[n * nslot + f] = o[n];
}

__device__ __forceinline__ long long wave_clock()
{
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int *p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

// Exchange words (the pencil schedule, cf_pencil.cuh): 64 bits per 32-bit
// part of a value (two parts for double), the part in the low half and a
// 32-bit tag naming the sweep in the high half, stored and loaded with
// relaxed 64-bit accesses.  A word either holds this sweep's value or shows
// that it does not yet, so a consumer polls the words themselves and its
// producer needs no fence and no flag.  The tag is 2 epoch (forward) or
// 2 epoch + 1 (backward), the epoch a device counter bumped once per call.
template <typename T>
struct wv_w {
    static constexpr int W = (int)(sizeof(T) / 4);
};

__device__ __forceinline__ void wv_st64(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long wv_ld64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void wv_put(unsigned long long *dst, float v, unsigned tag)
{
    wv_st64(dst, ((unsigned long long)tag << 32) | __float_as_uint(v));
}
__device__ __forceinline__ void wv_put(unsigned long long *dst, double v, unsigned tag)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    wv_st64(dst, ((unsigned long long)tag << 32) | (b & 0xffffffffull));
    wv_st64(dst + 1, ((unsigned long long)tag << 32) | (b >> 32));
}
__device__ __forceinline__ float wv_get(const unsigned *x, float) { return __uint_as_float(x[0]); }
__device__ __forceinline__ double wv_get(const unsigned *x, double)
{
    return __longlong_as_double((long long)(((unsigned long long)x[1] << 32) | x[0]));
}

// the epoch word after the claim counter and the error word
__device__ __forceinline__ int *wv_epoch(const wave_args &w, int nunits)
{
    return w.flags + nunits + 2;
}
__device__ __forceinline__ unsigned wv_tag(const wave_args &w, int nunits, bool fwd)
{
    return 2u * (unsigned)*wv_epoch(w, nunits) + (fwd ? 0u : 1u);
}

// one thread: the next epoch of the exchange tags
__global__ void k_lu_wave_epoch(wave_args w, int nunits)
{
    *wv_epoch(w, nunits) += 1;
}


// the same terms as tagged exchange words
template <typename T, bool UPPER>
__device__ __forceinline__ void wave_ghost_words(const cf_dims &d, const cf_lu_args &a, size_t qg, int dir,
                                                 const lu_den<T> &den, unsigned long long *face, int nslot, int f,
                                                 unsigned tag)
{
    const lstate<T> s = lu_state<T>(d, a, qg);
    const lsplit<T> A = wave_split<T>(d, a, qg, s, dir);
    T P[12], o[5];
    wave_split12<T, UPPER>(A, P);
    wave_scale<T>(P, den);
    const T zero[5] = {T(0), T(0), T(0), T(0), T(0)};
    if (UPPER) wave_upper_terms<T>(P, zero, den, o);
    else wave_lower_terms<T>(P, zero, den, o);
#pragma unroll
    for (int n = 0; n < 5; n++) wv_put(face + (n * nslot + f) * wv_w<T>::W, o[n], tag);
}

template <typename T>
__device__ __forceinline__ T ld_cg(const void *base, size_t q)
{
    return __ldcg(static_cast<const T *>(base) + q);
}

// Tile packs, one block (256 threads, one per cell) per tile, after
// k_lu_assemble (MR written).  Value m of the tile's cells is 256
// consecutive elements of the pack, so each thread stores its cell's values
// straight to HBM and every warp store is one contiguous 128-byte (FP64:
// 256-byte) row; no shared-memory staging limits the blocks per SM.  Also
// the terms of the ghost neighbours on the three lower faces of the domain.
// ASM: also the assembly of the tile's cells (lu_mr, MR written), which the
// wavefront then needs no separate pass for; the initial NL, NR of the
// assembly kernel are not formed (the sweeps overwrite every interior cell)
template <typename T, bool ASM>
__global__ void __launch_bounds__(256) k_lu_tile_pack(cf_lu_args a, wave_args w, T dt)
{
    const cf_dims &d = w.d;
    const int tile = blockIdx.x;
    int ta, tb, tc;
    wave_tile_coords(w, tile, ta, tb, tc);
    const int c = threadIdx.x;
    const int li = c / (WV_TJ * WV_TK), lj = (c / WV_TK) % WV_TJ, lk = c % WV_TK;
    const int i = 3 + ta * WV_TI + li, j = 2 + tb * WV_TJ + lj, k = 2 + tc * WV_TK + lk;
    const bool in = i <= d.gend && j <= d.ny && k <= d.nz;
    const lu_den<T> den[3] = {lu_den<T>(CF_DC(T, d, dXI)), lu_den<T>(CF_DC(T, d, dET)), lu_den<T>(CF_DC(T, d, dZT))};
    // value m of this cell at P[m * WV_CELLS] of the tile's pack
    T *P = static_cast<T *>(w.pack) + (size_t)tile * WV_CELLS * WV_PACK + c;
    lsplit<T> A[3];
    ldiag<T> g;
    size_t q = 0;
    T v[12];
    if (in) {
        q = d.ix(i, j, k);
        const lstate<T> s = lu_state<T>(d, a, q);
#pragma unroll
        for (int dir = 0; dir < 3; dir++) A[dir] = wave_split<T>(d, a, q, s, dir);
        g = lu_diag<T>(d, a, q, s, dt);
#pragma unroll
        for (int dir = 0; dir < 3; dir++) {
            wave_split12<T, false>(A[dir], v);
            wave_scale<T>(v, den[dir]);
            P[(39 + 2 * dir) * WV_CELLS] = v[0];       // p11
            P[(40 + 2 * dir) * WV_CELLS] = v[1];       // p22
#pragma unroll
            for (int m = 2; m < 12; m++) P[(6 + 10 * dir + m - 2) * WV_CELLS] = v[m];
            wave_split12<T, true>(A[dir], v);
            wave_scale<T>(v, den[dir]);
            P[(2 * dir) * WV_CELLS] = v[0];            // m11
            P[(2 * dir + 1) * WV_CELLS] = v[1];        // m22
        }
        P[36 * WV_CELLS] = g.d11; P[37 * WV_CELLS] = g.d22; P[38 * WV_CELLS] = g.d51;
        T MR[5];
        if (ASM) lu_mr<T>(d, a, i, j, k, q, dt, s, MR);
#pragma unroll
        for (int n = 0; n < 5; n++) {
            if (ASM) rhs_put<T>(a.MR[n], q, MR[n], a.f32_lu);
            else MR[n] = rhs_get<T>(a.MR[n], q, a.f32_lu);
            P[(45 + n) * WV_CELLS] = MR[n];
        }
    }
    if (in) {
        if (i == 3) wave_ghost_term<T, false>(d, a, q - d.plane(), 0, den[0], wave_face<T>(w, 0, tile), WV_FX,
                                              lj * WV_TK + lk);
        if (j == 2) wave_ghost_term<T, false>(d, a, q - (size_t)d.Zm, 1, den[1], wave_face<T>(w, 1, tile), WV_FY,
                                              li * WV_TK + lk);
        if (k == 2) wave_ghost_term<T, false>(d, a, q - 1, 2, den[2], wave_face<T>(w, 2, tile), WV_FZ,
                                              li * WV_TJ + lj);
    }
}

// the backward sweep's ghost terms on the three upper faces of the domain
// (a second launch: the forward sweep has consumed the face slots by then)
template <typename T>
__global__ void __launch_bounds__(256) k_lu_tile_ghost_upper(cf_lu_args a, wave_args w, cf_box b)
{
    const cf_dims &d = w.d;
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k);
    const int ci = i - 3, cj = j - 2, ck = k - 2;
    const int tile = ((ci / WV_TI) * w.ntj + cj / WV_TJ) * w.ntk + ck / WV_TK;
    const int li = ci % WV_TI, lj = cj % WV_TJ, lk = ck % WV_TK;
    const lu_den<T> dXI(CF_DC(T, d, dXI)), dET(CF_DC(T, d, dET)), dZT(CF_DC(T, d, dZT));
    if (i == d.gend) wave_ghost_term<T, true>(d, a, q + d.plane(), 0, dXI, wave_face<T>(w, 0, tile), WV_FX,
                                              lj * WV_TK + lk);
    if (j == d.ny) wave_ghost_term<T, true>(d, a, q + (size_t)d.Zm, 1, dET, wave_face<T>(w, 1, tile), WV_FY,
                                            li * WV_TK + lk);
    if (k == d.nz) wave_ghost_term<T, true>(d, a, q + 1, 2, dZT, wave_face<T>(w, 2, tile), WV_FZ, li * WV_TJ + lj);
}

constexpr int WV_WARPS = 4;                  // x terms, y terms, z terms, N
constexpr int WV_STEPS = WV_TI + WV_TJ + WV_TK - 2;

// shared memory of k_lu_wave, in elements of T
constexpr int WV_SM_PACK = WV_CELLS * WV_STAGE;
constexpr int WV_SM_IN = 15 * WV_CELLS;             // [3][5][cells] incoming terms
constexpr int WV_SM_N = 5 * WV_CELLS;               // [5][cells] this sweep's N
constexpr int WV_SM_NL = 5 * WV_CELLS;              // [5][cells] forward N (backward sweep input)
constexpr int WV_SM_OUT = 5 * (WV_FX + WV_FY + WV_FZ);
constexpr int WV_SM_TOTAL = WV_SM_PACK + WV_SM_IN + WV_SM_N + WV_SM_NL + WV_SM_OUT;

// The local-plane steps of one tile for the warp with role W: W = 0, 1, 2
// form the terms owed along x, y, z, W = 3 keeps N.  The role is a template
// parameter, so every offset and bound is a constant; the four warps meet
// at named barrier 1 once per step (every role takes the same L steps).
template <typename T, bool FWD, int W>
__device__ __forceinline__ void wave_steps(int L, bool full, int ti, int tj, int tk, const short (*s_cell)[32],
                                           const T *spack, T *sin, T *sN, const T *snl, T *sout,
                                           const lu_den<T> &dw, int lane)
{
    for (int s = 0; s < L; s++) {
        const int l = FWD ? s : L - 1 - s;
        const int c = s_cell[l][lane];
        const int li = c / (WV_TJ * WV_TK), lj = (c / WV_TK) % WV_TJ, lk = c % WV_TK;
        if (c >= 0 && (full || (li < ti && lj < tj && lk < tk))) {
            const T *P = spack + c;                    // value m at P[m * WV_CELLS]
            T S[5], N[5];
#pragma unroll
            for (int n = 0; n < 5; n++)
                S[n] = (sin[(0 * 5 + n) * WV_CELLS + c] + sin[(1 * 5 + n) * WV_CELLS + c]) +
                       sin[(2 * 5 + n) * WV_CELLS + c];
            // staged window: forward values 6..49 at 0..43, backward 0..38
            constexpr int wo = FWD ? WV_FWD0 : 0;
            const T d11 = P[(36 - wo) * WV_CELLS], d22 = P[(37 - wo) * WV_CELLS], d51 = P[(38 - wo) * WV_CELLS];
            if (FWD) {
                const T r0 = P[(45 - wo) * WV_CELLS] - S[0];
                N[0] = d11 * r0;
                N[1] = d22 * (P[(46 - wo) * WV_CELLS] - S[1]);
                N[2] = d22 * (P[(47 - wo) * WV_CELLS] - S[2]);
                N[3] = d22 * (P[(48 - wo) * WV_CELLS] - S[3]);
                N[4] = d51 * r0 + d22 * (P[(49 - wo) * WV_CELLS] - S[4]);
            } else {
                N[0] = snl[0 * WV_CELLS + c] - d11 * S[0];
                N[1] = snl[1 * WV_CELLS + c] - d22 * S[1];
                N[2] = snl[2 * WV_CELLS + c] - d22 * S[2];
                N[3] = snl[3 * WV_CELLS + c] - d22 * S[3];
                N[4] = snl[4 * WV_CELLS + c] - (d51 * S[0] + d22 * S[4]);
            }
            if (W == 3) {
#pragma unroll
                for (int n = 0; n < 5; n++) sN[n * WV_CELLS + c] = N[n];
            } else {
                // the terms owed to the next cell along direction W
                // this direction's split: p11 p22 (forward) or m11 m22
                // (backward), then p12 .. p54
                T o[5], cw[12];
                cw[0] = P[((FWD ? 39 : 0) + 2 * W - wo) * WV_CELLS];
                cw[1] = P[((FWD ? 40 : 1) + 2 * W - wo) * WV_CELLS];
#pragma unroll
                for (int m = 2; m < 12; m++) cw[m] = P[(6 + 10 * W + m - 2 - wo) * WV_CELLS];
                if (FWD) wave_lower_terms<T>(cw, N, dw, o);
                else wave_upper_terms<T>(cw, N, dw, o);
                constexpr int cstep = W == 0 ? WV_TJ * WV_TK : W == 1 ? WV_TK : 1;
                const int lc = W == 0 ? li : W == 1 ? lj : lk;
                const int tcw = W == 0 ? ti : W == 1 ? tj : tk;
                if (FWD ? lc + 1 < tcw : lc >= 1) {
                    const int cn = FWD ? c + cstep : c - cstep;
#pragma unroll
                    for (int n = 0; n < 5; n++) sin[(W * 5 + n) * WV_CELLS + cn] = o[n];
                } else {
                    // leaves the tile: shared face buffer of this direction
                    constexpr int off = W == 0 ? 0 : W == 1 ? 5 * WV_FX : 5 * (WV_FX + WV_FY);
                    constexpr int ns = W == 0 ? WV_FX : W == 1 ? WV_FY : WV_FZ;
                    const int f = W == 0 ? lj * WV_TK + lk : W == 1 ? li * WV_TK + lk : li * WV_TJ + lj;
#pragma unroll
                    for (int n = 0; n < 5; n++) sout[off + n * ns + f] = o[n];
                }
            }
        }
        asm volatile("bar.sync 1, %0;" :: "n"(32 * WV_WARPS) : "memory");
    }
}

// FWD: forward sweep (NL), else backward (NR).  Four warps per block: all
// four form the cell's N from the incoming terms; warps 0, 1, 2 then form
// the terms owed along x, y, z and warp 3 keeps N.  Terms for cells of the
// tile go to shared memory, terms for the next tile to a shared face buffer
// that is copied to that tile's face slot (coalesced) before the done flag;
// N goes to HBM after the flag.
template <typename T, bool FWD>
__global__ void __launch_bounds__(32 * WV_WARPS) k_lu_wave(cf_lu_args a, wave_args w)
{
    extern __shared__ __align__(128) unsigned char wave_smem[];
    T *spack = reinterpret_cast<T *>(wave_smem);
    T *sin = spack + WV_SM_PACK;
    T *sN = sin + WV_SM_IN;
    T *snl = sN + WV_SM_N;
    T *sout = snl + WV_SM_NL;                                      // x [5][64], y [5][32], z [5][32]
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ int s_slot;
    __shared__ short s_cell[WV_STEPS][32];                         // local plane l, lane -> cell (-1: none)
    const cf_dims &d = w.d;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned bar = smem_u32(&mbar);
    for (int e = tid; e < WV_STEPS * 32; e += 32 * WV_WARPS) {
        int li, lj, lk;
        const int l = e / 32, t = e % 32;
        s_cell[l][t] = wave_cell(l, t, WV_TI, WV_TJ, WV_TK, li, lj, lk)
                           ? (short)((li * WV_TJ + lj) * WV_TK + lk) : (short)-1;
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_slot = atomicAdd(w.counter, 1);
    }
    __syncthreads();
    int slot = s_slot;
    __syncthreads();
    unsigned phase = 0;
    const lu_den<T> dw(T(warp == 0 ? d.dXI : warp == 1 ? d.dET : d.dZT));   // this warp's direction
    // the sweep's window of each tile pack: forward values 6..49, backward 0..38
    const unsigned pbytes = (unsigned)((FWD ? WV_STAGE : 39) * WV_CELLS * sizeof(T));
    const unsigned nbytes = (unsigned)(WV_SM_NL * sizeof(T));
    const T *packsrc = static_cast<const T *>(w.pack) + (FWD ? WV_FWD0 * WV_CELLS : 0);
    while (slot < w.ntiles) {
        const int tile = w.order[FWD ? slot : w.ntiles - 1 - slot];
        int ta, tb, tc;
        wave_tile_coords(w, tile, ta, tb, tc);
        const int i0 = 3 + ta * WV_TI, j0 = 2 + tb * WV_TJ, k0 = 2 + tc * WV_TK;
        const int ti = min(WV_TI, d.gend - i0 + 1), tj = min(WV_TJ, d.ny - j0 + 1), tk = min(WV_TK, d.nz - k0 + 1);
        long long *tr = w.trace ? w.trace + 4 * (size_t)tile : nullptr;
        if (tr && tid == 0) tr[0] = wave_clock();
        // stage the tile's coefficients (and, backward, the forward N): the
        // barrier and the proxy fence order the previous tile's reads of
        // these buffers before the async-proxy writes
        if (tid == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const T *src = packsrc + (size_t)tile * WV_CELLS * WV_PACK;
            const unsigned total = FWD ? pbytes : pbytes + nbytes;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(total) : "memory");
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                         :: "r"(smem_u32(spack)), "l"(src), "r"(pbytes), "r"(bar) : "memory");
            if (!FWD) {
                const T *nsrc = static_cast<const T *>(w.nl) + (size_t)tile * WV_SM_NL;
                asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                             :: "r"(smem_u32(snl)), "l"(nsrc), "r"(nbytes), "r"(bar) : "memory");
            }
        }
        // wait for the neighbour tiles (threads 0..2, one direction each)
        if (tid < 3) {
            int na = ta, nb = tb, nc = tc;
            const int step = FWD ? -1 : 1;
            if (tid == 0) na += step;
            if (tid == 1) nb += step;
            if (tid == 2) nc += step;
            if (na >= 0 && na < w.nti && nb >= 0 && nb < w.ntj && nc >= 0 && nc < w.ntk) {
                const int *f = w.flags + (na * w.ntj + nb) * w.ntk + nc;
                unsigned it = 0;
                while (ld_acquire(f) == 0) {
                    if (++it > w.dep_limit) {
                        atomicOr(w.err, 1);
                        break;
                    }
                    // after any wait has run out, no other wait spins
                    if ((it & 1023u) == 0 && ld_acquire(w.err) != 0) break;
                    __nanosleep(20);
                }
            }
        }
        __syncthreads();
        // incoming terms of the tile's three entry faces, one coalesced round:
        // threads 0..63 the x face, 64..95 the y face, 96..127 the z face
        {
            const int fi = FWD ? 0 : ti - 1, fj = FWD ? 0 : tj - 1, fk = FWD ? 0 : tk - 1;
            int dir, f, cc = -1, nslot;
            if (tid < WV_FX) {
                dir = 0; f = tid; nslot = WV_FX;
                const int lj = f / WV_TK, lk = f % WV_TK;
                if (lj < tj && lk < tk) cc = (fi * WV_TJ + lj) * WV_TK + lk;
            } else if (tid < WV_FX + WV_FY) {
                dir = 1; f = tid - WV_FX; nslot = WV_FY;
                const int li = f / WV_TK, lk = f % WV_TK;
                if (li < ti && lk < tk) cc = (li * WV_TJ + fj) * WV_TK + lk;
            } else {
                dir = 2; f = tid - WV_FX - WV_FY; nslot = WV_FZ;
                const int li = f / WV_TJ, lj = f % WV_TJ;
                if (li < ti && lj < tj) cc = (li * WV_TJ + lj) * WV_TK + fk;
            }
            if (cc >= 0) {
                const T *src = wave_face<T>(w, dir, tile);
                T v[5];
#pragma unroll
                for (int n = 0; n < 5; n++) v[n] = __ldcg(src + n * nslot + f);
#pragma unroll
                for (int n = 0; n < 5; n++) sin[(dir * 5 + n) * WV_CELLS + cc] = v[n];
            }
        }
        if (tr && tid == 0) tr[1] = wave_clock();
        // claim the next tile now; the answer is needed only after this one
        if (tid == 0) s_slot = atomicAdd(w.counter, 1);
        // the staged data has landed
        {
            unsigned it = 0, done = 0;
            for (;;) {
                asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                             " selp.u32 %0, 1, 0, p;\n}" : "=r"(done) : "r"(bar), "r"(phase) : "memory");
                if (done) break;
                if (++it > WV_SPIN_LIMIT) {
                    if (tid == 0) atomicOr(w.err, 2);
                    break;
                }
            }
            phase ^= 1;
        }
        __syncthreads();
        if (tr && tid == 0) tr[2] = wave_clock();
        const int L = ti + tj + tk - 2;
        const bool full = ti == WV_TI && tj == WV_TJ && tk == WV_TK;
        switch (warp) {
        case 0: wave_steps<T, FWD, 0>(L, full, ti, tj, tk, s_cell, spack, sin, sN, snl, sout, dw, lane); break;
        case 1: wave_steps<T, FWD, 1>(L, full, ti, tj, tk, s_cell, spack, sin, sN, snl, sout, dw, lane); break;
        case 2: wave_steps<T, FWD, 2>(L, full, ti, tj, tk, s_cell, spack, sin, sN, snl, sout, dw, lane); break;
        default: wave_steps<T, FWD, 3>(L, full, ti, tj, tk, s_cell, spack, sin, sN, snl, sout, dw, lane); break;
        }
        // terms for the next tiles into their entry-face slots, then the flag
        {
            int dir, f, ns, off;
            if (tid < WV_FX) { dir = 0; f = tid; ns = WV_FX; off = 0; }
            else if (tid < WV_FX + WV_FY) { dir = 1; f = tid - WV_FX; ns = WV_FY; off = 5 * WV_FX; }
            else { dir = 2; f = tid - WV_FX - WV_FY; ns = WV_FZ; off = 5 * (WV_FX + WV_FY); }
            const int tcoord = dir == 0 ? ta : dir == 1 ? tb : tc;
            const int tcount = dir == 0 ? w.nti : dir == 1 ? w.ntj : w.ntk;
            if (FWD ? tcoord + 1 < tcount : tcoord >= 1) {
                const int ts = dir == 0 ? w.ntj * w.ntk : dir == 1 ? w.ntk : 1;
                T *dst = wave_face<T>(w, dir, FWD ? tile + ts : tile - ts);
#pragma unroll
                for (int n = 0; n < 5; n++) dst[n * ns + f] = sout[off + n * ns + f];
            }
        }
        __threadfence();
        __syncthreads();
        if (tid == 0) st_release(w.flags + tile, 1);
        if (tr && tid == 0) tr[3] = wave_clock();
        // N of the tile to HBM (read only by later launches)
        for (int v = tid; v < 5 * WV_CELLS; v += 32 * WV_WARPS) {
            const int n = v / WV_CELLS, c = v % WV_CELLS;
            const int li = c / (WV_TJ * WV_TK), lj = (c / WV_TK) % WV_TJ, lk = c % WV_TK;
            const T x = sN[v];
            if (FWD) static_cast<T *>(w.nl)[(size_t)tile * WV_SM_NL + v] = x;
            if (li < ti && lj < tj && lk < tk) {
                const size_t q = d.ix(i0 + li, j0 + lj, k0 + lk);
                // (the FP32 step driver reads the forward N from the tile
                // layout only)
                if (FWD && !(sizeof(T) == 4 && cf_step_layout)) rhs_put<T>(a.NL[n], q, x, a.f32_lu);
                else rhs_put<T>(a.NR[n], q, x, a.f32_lu);
            }
        }
        slot = s_slot;
        __syncthreads();
    }
    if (tid == 0) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" :: "r"(bar) : "memory");
}

}  // namespace CF_NS
