// Hyperplane LU-SGS sweeps as pencils (Dual_time_stepping.cpp:563-1250).
//
// A pencil is a 4 x 8 block of (j, k) columns through every x plane of the
// interior; one warp sweeps it, lane lj*8 + lk owning column (j0+lj, k0+lk).
// At step s of the forward sweep the lane computes cell i = 3 + s - lj - lk
// (when that cell exists), so every step of the warp is one local
// hyperplane of the pencil and consecutive steps of a lane walk its column
// along x.  The three terms a cell needs arrive
//   x: from the lane's own previous step (a register),
//   y: from lane (lj-1, lk) of the previous step (a warp shuffle),
//   z: from lane (lj, lk-1) of the previous step (a warp shuffle),
// and across the pencil's lower faces from the neighbour pencils through
// exchange words in HBM, whose producer is 3 (y) or 7 (z) steps ahead of
// the consumer.  An exchange word is 64 bits: 32 bits of the value and a
// 32-bit tag naming the sweep (an epoch counter in device memory, bumped
// once per call), stored and loaded with relaxed 64-bit accesses, so a word
// either holds this sweep's value or shows that it does not yet: no fence
// and no progress flag is needed.  A warp loads the words of the next
// PC_PUB steps one block ahead into registers and, at the block's start,
// re-reads only those whose tag was not yet this sweep's (bounded).  So
// the sweep's critical path is about X_out + (3 + 2 PC_PUB) npj +
// (7 + 2 PC_PUB) npk steps of one cell each, against (tiles along the
// diagonal) x (local planes per tile) for 4 x 8 x 8 tiles.
// The backward sweep runs the same steps in reverse with the upper terms.
//
// Every cell is computed from exactly the inputs of the reference's
// plane-ordered loop, with the arithmetic of the tiled wavefront
// (cf_wave.cuh), so all schedules give the same bits.
//
// Coefficients: one pack per pencil, plane-major ([plane][value][lane],
// value order of cf_wave.cuh's tile pack), so the 32 lanes of a step read
// one contiguous block; a lane stages the next PC_DEPTH planes with bulk
// async copies (cp.async.bulk, one mbarrier per ring slot) while it
// computes.  Every wait is bounded; a wait that runs out sets the error
// word the host reads and the warp goes on.
#pragma once
#include "cf_wave.cuh"

namespace CF_NS {

constexpr int PC_TJ = CF_PENCIL_TJ, PC_TK = CF_PENCIL_TK;
constexpr int PC_SKEW = PC_TJ - 1 + PC_TK - 1;      // largest lj + lk
constexpr int PC_DEPTH = 4;                          // staged planes per warp
constexpr int PC_PUB = CF_PENCIL_PUB;

template <typename T>
struct pc_geom {
    static constexpr int WARPS = sizeof(T) == 4 ? 4 : 2;   // pencils per block
};

// values a sweep stages per plane: forward pack values 6..49; backward
// 0..38 and the forward N (5)
template <bool FWD>
struct pc_stage {
    static constexpr int NV = FWD ? WV_STAGE : 39;
    static constexpr int NS = NV + (FWD ? 0 : 5);
    static constexpr int WO = FWD ? WV_FWD0 : 0;     // first pack value staged
};

template <typename T>
constexpr size_t pc_smem_bytes(bool fwd)
{
    return (size_t)pc_geom<T>::WARPS * PC_DEPTH * (fwd ? pc_stage<true>::NS : pc_stage<false>::NS) * 32 * sizeof(T);
}

template <typename T>
__device__ __forceinline__ T *pc_pack(const wave_args &w, int pencil, int p)
{
    return static_cast<T *>(w.pack) + ((size_t)pencil * w.nplanes + p) * WV_PACK * 32;
}
template <typename T>
__device__ __forceinline__ T *pc_nl(const wave_args &w, int pencil, int p)
{
    return static_cast<T *>(w.nl) + ((size_t)pencil * w.nplanes + p) * 5 * 32;
}
template <typename T>
__device__ __forceinline__ T *pc_xg(const wave_args &w, int pencil)
{
    return static_cast<T *>(w.xg) + (size_t)pencil * 5 * 32;
}
// exchange words: per pencil and x cell [5][8 (lk)] (y face) or [5][4 (lj)]
// (z face) values of PC_W words each
template <typename T>
struct pc_w {
    static constexpr int W = wv_w<T>::W;
};
template <typename T>
__device__ __forceinline__ unsigned long long *pc_yex(const wave_args &w, int pencil, int ci)
{
    return static_cast<unsigned long long *>(w.yex) + ((size_t)pencil * w.d.X_out + ci) * 5 * PC_TK * pc_w<T>::W;
}
template <typename T>
__device__ __forceinline__ unsigned long long *pc_zex(const wave_args &w, int pencil, int ci)
{
    return static_cast<unsigned long long *>(w.zex) + ((size_t)pencil * w.d.X_out + ci) * 5 * PC_TJ * pc_w<T>::W;
}


// Pencil packs: one block of 256 threads per 8 x-planes of a pencil (cell
// li*32 + lane), the values formed as for the tile pack in shared memory,
// then written plane-major; and the terms of the ghost cells below the
// domain's lower faces.  ASM: also the assembly (lu_mr, MR written).
template <typename T, bool ASM>
__global__ void __launch_bounds__(256) k_lu_pencil_pack(cf_lu_args a, wave_args w, T dt)
{
    extern __shared__ __align__(128) unsigned char pcp_smem[];
    T *sp = reinterpret_cast<T *>(pcp_smem);     // [WV_PACK][256]
    const cf_dims &d = w.d;
    const int nchunk = (d.X_out + 7) / 8;
    const int pencil = blockIdx.x / nchunk, chunk = blockIdx.x % nchunk;
    const int pb = pencil / w.npk, pk = pencil % w.npk;
    const int c = threadIdx.x, li = c >> 5, lane = c & 31, lj = lane >> 3, lk = lane & 7;
    const int i = 3 + chunk * 8 + li, j = 2 + pb * PC_TJ + lj, k = 2 + pk * PC_TK + lk;
    const bool in = i <= d.gend && j <= d.ny && k <= d.nz;
    const lu_den<T> den[3] = {lu_den<T>(CF_DC(T, d, dXI)), lu_den<T>(CF_DC(T, d, dET)), lu_den<T>(CF_DC(T, d, dZT))};
    T *P = sp + c;
    size_t q = 0;
    if (in) {
        q = d.ix(i, j, k);
        const lstate<T> s = lu_state<T>(d, a, q);
        T v[12];
#pragma unroll
        for (int dir = 0; dir < 3; dir++) {
            const lsplit<T> A = wave_split<T>(d, a, q, s, dir);
            wave_split12<T, false>(A, v);
            wave_scale<T>(v, den[dir]);
            P[(39 + 2 * dir) * 256] = v[0];
            P[(40 + 2 * dir) * 256] = v[1];
#pragma unroll
            for (int m = 2; m < 12; m++) P[(6 + 10 * dir + m - 2) * 256] = v[m];
            wave_split12<T, true>(A, v);
            wave_scale<T>(v, den[dir]);
            P[(2 * dir) * 256] = v[0];
            P[(2 * dir + 1) * 256] = v[1];
        }
        const ldiag<T> g = lu_diag<T>(d, a, q, s, dt);
        P[36 * 256] = g.d11; P[37 * 256] = g.d22; P[38 * 256] = g.d51;
        T MR[5];
        if (ASM) lu_mr<T>(d, a, i, j, k, q, dt, s, MR);
#pragma unroll
        for (int n = 0; n < 5; n++) {
            if (ASM) rhs_put<T>(a.MR[n], q, MR[n], a.f32_lu);
            else MR[n] = rhs_get<T>(a.MR[n], q, a.f32_lu);
            P[(45 + n) * 256] = MR[n];
        }
        if (i == 3) wave_ghost_term<T, false>(d, a, q - d.plane(), 0, den[0], pc_xg<T>(w, pencil), 32, lane);
        if (j == 2) wave_ghost_words<T, false>(d, a, q - (size_t)d.Zm, 1, den[1], pc_yex<T>(w, pencil, i - 3), PC_TK,
                                             lk, wv_tag(w, w.npencils, true));
        if (k == 2) wave_ghost_words<T, false>(d, a, q - 1, 2, den[2], pc_zex<T>(w, pencil, i - 3), PC_TJ, lj,
                                             wv_tag(w, w.npencils, true));
    }
    __syncthreads();
    // plane-major write: warp wp takes planes p0 + wp, p0 + wp + 8, ...;
    // lane's cell of plane p is li = p - p0 - lj - lk of this chunk
    const int p0 = chunk * 8, wp = c >> 5;
    for (int pp = wp; pp < 8 + PC_SKEW; pp += 8) {
        const int p = p0 + pp, lc = pp - lj - lk;
        if (p >= w.nplanes || lc < 0 || lc >= 8) continue;
        if (3 + chunk * 8 + lc > d.gend || j > d.ny || k > d.nz) continue;
        T *dst = pc_pack<T>(w, pencil, p) + lane;
        const T *src = sp + lc * 32 + lane;
#pragma unroll 10
        for (int m = 0; m < WV_PACK; m++) dst[m * 32] = src[m * 256];
    }
}

// the backward sweep's ghost terms above the domain's upper faces
template <typename T>
__global__ void __launch_bounds__(256) k_lu_pencil_ghost_upper(cf_lu_args a, wave_args w, cf_box b)
{
    const cf_dims &d = w.d;
    CF_BOX_INDEX(b, i, j, k);
    const size_t q = d.ix(i, j, k);
    const int cj = j - 2, ck = k - 2;
    const int pencil = (cj / PC_TJ) * w.npk + ck / PC_TK, lj = cj % PC_TJ, lk = ck % PC_TK;
    const lu_den<T> dXI(CF_DC(T, d, dXI)), dET(CF_DC(T, d, dET)), dZT(CF_DC(T, d, dZT));
    if (i == d.gend) wave_ghost_term<T, true>(d, a, q + d.plane(), 0, dXI, pc_xg<T>(w, pencil), 32, lj * PC_TK + lk);
    if (j == d.ny) wave_ghost_words<T, true>(d, a, q + (size_t)d.Zm, 1, dET, pc_yex<T>(w, pencil, i - 3), PC_TK, lk,
                                           wv_tag(w, w.npencils, false));
    if (k == d.nz) wave_ghost_words<T, true>(d, a, q + 1, 2, dZT, pc_zex<T>(w, pencil, i - 3), PC_TJ, lj,
                                           wv_tag(w, w.npencils, false));
}

// the five terms a cell owes its neighbour along direction W, from the
// direction's 12 staged split values (P: this lane's staged plane)
template <typename T, bool FWD, int WO, int W>
__device__ __forceinline__ void pc_terms(const T *P, const T *N, const lu_den<T> &den, T *o)
{
    T cw[12];
    cw[0] = P[((FWD ? 39 : 0) + 2 * W - WO) * 32];
    cw[1] = P[((FWD ? 40 : 1) + 2 * W - WO) * 32];
#pragma unroll
    for (int m = 2; m < 12; m++) cw[m] = P[(6 + 10 * W + m - 2 - WO) * 32];
    if (FWD) wave_lower_terms<T>(cw, N, den, o);
    else wave_upper_terms<T>(cw, N, den, o);
}

// the exchange words one lane handles per block of PC_PUB steps
template <typename T>
struct pc_pre {
    static constexpr int WORDS = PC_PUB * 5 * (PC_TK + PC_TJ) * pc_w<T>::W;   // per block and warp
    static constexpr int PER_LANE = (WORDS + 31) / 32;
};

// address of exchange word e of the block starting at step s0 (null when the
// word is not read: past the last step, or no such cell)
template <typename T, bool FWD>
__device__ __forceinline__ const unsigned long long *pc_word_addr(const wave_args &w, int pencil, int s0, int e,
                                                                  int NP, int tj, int tk)
{
    constexpr int W = pc_w<T>::W, C = PC_TK + PC_TJ;
    const int tt = e / (5 * C * W), r = e % (5 * C * W);
    const int n = r / (C * W), c = (r / W) % C, k = r % W;
    const int st = s0 + tt;
    if (st >= NP) return nullptr;
    const int p = FWD ? st : NP - 1 - st;
    const int ljy = FWD ? 0 : tj - 1, lkz = FWD ? 0 : tk - 1;
    if (c < PC_TK) {
        const int i = 3 + p - ljy - c;
        if (c >= tk || i < 3 || i > w.d.gend) return nullptr;
        return pc_yex<T>(w, pencil, i - 3) + (n * PC_TK + c) * W + k;
    }
    const int lj2 = c - PC_TK, i = 3 + p - lj2 - lkz;
    if (lj2 >= tj || i < 3 || i > w.d.gend) return nullptr;
    return pc_zex<T>(w, pencil, i - 3) + (n * PC_TJ + lj2) * W + k;
}

template <typename T, bool FWD>
__global__ void __launch_bounds__(32 * pc_geom<T>::WARPS) k_lu_pencil(cf_lu_args a, wave_args w)
{
    constexpr int NV = pc_stage<FWD>::NV, NS = pc_stage<FWD>::NS, WO = pc_stage<FWD>::WO;
    constexpr int WARPS = pc_geom<T>::WARPS, W = pc_w<T>::W, C = PC_TK + PC_TJ;
    constexpr int NPRE = pc_pre<T>::PER_LANE, WORDS = pc_pre<T>::WORDS;
    extern __shared__ __align__(128) unsigned char pc_smem[];
    __shared__ __align__(8) unsigned long long mbar[WARPS][PC_DEPTH];
    // this block's incoming face terms: [step][n][8 y slots (lk), 4 z slots (lj)][word]
    __shared__ unsigned xch[WARPS][PC_PUB][5][C][W];
    const cf_dims &d = w.d;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int lj = lane >> 3, lk = lane & 7;
    T *ring = reinterpret_cast<T *>(pc_smem) + (size_t)warp * PC_DEPTH * NS * 32;
    if (lane == 0) {
        for (int r = 0; r < PC_DEPTH; r++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&mbar[warp][r])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    const lu_den<T> den[3] = {lu_den<T>(CF_DC(T, d, dXI)), lu_den<T>(CF_DC(T, d, dET)), lu_den<T>(CF_DC(T, d, dZT))};
    const int NP = w.nplanes;
    const unsigned tag = wv_tag(w, w.npencils, FWD);
    const unsigned pbytes = (unsigned)(NV * 32 * sizeof(T)), nbytes = (unsigned)(5 * 32 * sizeof(T));
    unsigned gs = 0;                       // this warp's steps over all its pencils (ring slot and phase)
    int slot = 0;
    if (lane == 0) slot = atomicAdd(w.counter, 1);
    slot = __shfl_sync(0xffffffffu, slot, 0);
    while (slot < w.npencils) {
        const int pencil = w.order[FWD ? slot : w.npencils - 1 - slot];
        const int pb = pencil / w.npk, pk = pencil % w.npk;
        const int j0 = 2 + pb * PC_TJ, k0 = 2 + pk * PC_TK;
        const int tj = min(PC_TJ, d.ny - j0 + 1), tk = min(PC_TK, d.nz - k0 + 1);
        const bool lane_ok = lj < tj && lk < tk;
        const int j = j0 + lj, k = k0 + lk;
        // the neighbour pencils this pencil writes to
        const int yto = FWD ? (pb + 1 < w.npj ? pencil + w.npk : -1) : (pb > 0 ? pencil - w.npk : -1);
        const int zto = FWD ? (pk + 1 < w.npk ? pencil + 1 : -1) : (pk > 0 ? pencil - 1 : -1);
        const bool yedge_in = FWD ? lj == 0 : lj == tj - 1, zedge_in = FWD ? lk == 0 : lk == tk - 1;
        const bool yedge_out = FWD ? lj == tj - 1 : lj == 0, zedge_out = FWD ? lk == tk - 1 : lk == 0;
        // stage the first planes
        auto issue = [&](int s, unsigned g) {
            const int p = FWD ? s : NP - 1 - s;
            T *dst = ring + (g % PC_DEPTH) * NS * 32;
            const unsigned bar = smem_u32(&mbar[warp][g % PC_DEPTH]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                         :: "r"(bar), "r"(FWD ? pbytes : pbytes + nbytes) : "memory");
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                         :: "r"(smem_u32(dst)), "l"(pc_pack<T>(w, pencil, p) + WO * 32), "r"(pbytes), "r"(bar)
                         : "memory");
            if (!FWD)
                asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                             :: "r"(smem_u32(dst + NV * 32)), "l"(pc_nl<T>(w, pencil, p)), "r"(nbytes), "r"(bar)
                             : "memory");
        };
        if (lane == 0)
            for (int s = 0; s < PC_DEPTH && s < NP; s++) issue(s, gs + s);
        // optional trace: the claim, then the end of each block's wait
        long long *tr = w.trace ? w.trace + (size_t)pencil * ((NP + PC_PUB - 1) / PC_PUB + 1) : nullptr;
        if (tr && lane == 0) tr[0] = wave_clock();
        // the exchange words of the first block
        unsigned long long pre[NPRE];
#pragma unroll
        for (int m = 0; m < NPRE; m++) {
            const int e = lane + 32 * m;
            const unsigned long long *ad = e < WORDS ? pc_word_addr<T, FWD>(w, pencil, 0, e, NP, tj, tk) : nullptr;
            pre[m] = ad ? wv_ld64(ad) : 0ull;
        }
        T xo[5], yo[5], zo[5];
#pragma unroll
        for (int n = 0; n < 5; n++) xo[n] = yo[n] = zo[n] = T(0);
        for (int s = 0; s < NP; s++, gs++) {
            const int p = FWD ? s : NP - 1 - s;
            const int i = 3 + p - lj - lk;
            const bool valid = lane_ok && i >= 3 && i <= d.gend;
            // terms of the previous step from the neighbouring lanes
            T yin[5], zin[5];
#pragma unroll
            for (int n = 0; n < 5; n++) {
                yin[n] = FWD ? __shfl_up_sync(0xffffffffu, yo[n], PC_TK) : __shfl_down_sync(0xffffffffu, yo[n], PC_TK);
                zin[n] = FWD ? __shfl_up_sync(0xffffffffu, zo[n], 1) : __shfl_down_sync(0xffffffffu, zo[n], 1);
            }
            const int t = s % PC_PUB;
            if (t == 0) {
                // this block's words: re-read those not yet of this sweep
                // (bounded), then request the next block's
#pragma unroll
                for (int m = 0; m < NPRE; m++) {
                    const int e = lane + 32 * m;
                    if (e >= WORDS) continue;
                    const unsigned long long *ad = pc_word_addr<T, FWD>(w, pencil, s, e, NP, tj, tk);
                    unsigned v = 0;
                    if (ad) {
                        unsigned it = 0;
                        while ((unsigned)(pre[m] >> 32) != tag) {
                            if (++it > w.dep_limit) {
                                atomicOr(w.err, 1);
                                break;
                            }
                            if ((it & 1023u) == 0 && ld_acquire(w.err) != 0) break;
                            __nanosleep(20);
                            pre[m] = wv_ld64(ad);
                        }
                        v = (unsigned)(pre[m] & 0xffffffffull);
                    }
                    (&xch[warp][0][0][0][0])[e] = v;
                }
                if (tr && lane == 0) tr[1 + s / PC_PUB] = wave_clock();
#pragma unroll
                for (int m = 0; m < NPRE; m++) {
                    const int e = lane + 32 * m;
                    const unsigned long long *ad =
                        e < WORDS ? pc_word_addr<T, FWD>(w, pencil, s + PC_PUB, e, NP, tj, tk) : nullptr;
                    pre[m] = ad ? wv_ld64(ad) : 0ull;
                }
                __syncwarp();
            }
            // this step's plane has landed
            {
                const unsigned bar = smem_u32(&mbar[warp][gs % PC_DEPTH]), phase = (gs / PC_DEPTH) & 1u;
                unsigned it = 0, done = 0;
                for (;;) {
                    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                                 " selp.u32 %0, 1, 0, p;\n}" : "=r"(done) : "r"(bar), "r"(phase) : "memory");
                    if (done) break;
                    if (++it > WV_SPIN_LIMIT) {
                        if (lane == 0) atomicOr(w.err, 2);
                        break;
                    }
                }
            }
            if (valid) {
                const int ci = i - 3;
                T xin[5];
                const bool xfirst = FWD ? i == 3 : i == d.gend;
                if (xfirst) {
                    const T *g = pc_xg<T>(w, pencil);
#pragma unroll
                    for (int n = 0; n < 5; n++) xin[n] = __ldcg(g + n * 32 + lane);
                } else {
#pragma unroll
                    for (int n = 0; n < 5; n++) xin[n] = xo[n];
                }
                if (yedge_in) {
#pragma unroll
                    for (int n = 0; n < 5; n++) yin[n] = wv_get(xch[warp][t][n][lk], T(0));
                }
                if (zedge_in) {
#pragma unroll
                    for (int n = 0; n < 5; n++) zin[n] = wv_get(xch[warp][t][n][PC_TK + lj], T(0));
                }
                const T *P = ring + (gs % PC_DEPTH) * NS * 32 + lane;   // value m at P[(m - WO) * 32]
                T S[5], N[5];
#pragma unroll
                for (int n = 0; n < 5; n++) S[n] = (xin[n] + yin[n]) + zin[n];
                const T d11 = P[(36 - WO) * 32], d22 = P[(37 - WO) * 32], d51 = P[(38 - WO) * 32];
                if (FWD) {
                    const T r0 = P[(45 - WO) * 32] - S[0];
                    N[0] = d11 * r0;
                    N[1] = d22 * (P[(46 - WO) * 32] - S[1]);
                    N[2] = d22 * (P[(47 - WO) * 32] - S[2]);
                    N[3] = d22 * (P[(48 - WO) * 32] - S[3]);
                    N[4] = d51 * r0 + d22 * (P[(49 - WO) * 32] - S[4]);
                } else {
                    const T *nl = P + NV * 32;
                    N[0] = nl[0 * 32] - d11 * S[0];
                    N[1] = nl[1 * 32] - d22 * S[1];
                    N[2] = nl[2 * 32] - d22 * S[2];
                    N[3] = nl[3 * 32] - d22 * S[3];
                    N[4] = nl[4 * 32] - (d51 * S[0] + d22 * S[4]);
                }
                // the terms owed along x, y, z
                pc_terms<T, FWD, WO, 0>(P, N, den[0], xo);
                pc_terms<T, FWD, WO, 1>(P, N, den[1], yo);
                pc_terms<T, FWD, WO, 2>(P, N, den[2], zo);
                // terms leaving the pencil: tagged words in the next pencil's slots
                if (yedge_out && yto >= 0) {
                    unsigned long long *e = pc_yex<T>(w, yto, ci);
#pragma unroll
                    for (int n = 0; n < 5; n++) wv_put(e + (n * PC_TK + lk) * W, yo[n], tag);
                }
                if (zedge_out && zto >= 0) {
                    unsigned long long *e = pc_zex<T>(w, zto, ci);
#pragma unroll
                    for (int n = 0; n < 5; n++) wv_put(e + (n * PC_TJ + lj) * W, zo[n], tag);
                }
                const size_t q = d.ix(i, j, k);
                if (FWD) {
                    T *nlp = pc_nl<T>(w, pencil, p) + lane;
#pragma unroll
                    for (int n = 0; n < 5; n++) nlp[n * 32] = N[n];
                } else {
#pragma unroll
                    for (int n = 0; n < 5; n++) rhs_put<T>(a.NR[n], q, N[n], a.f32_lu);
                }
            } else {
#pragma unroll
                for (int n = 0; n < 5; n++) xo[n] = yo[n] = zo[n] = T(0);
            }
            // every lane has read the ring slot and this step's face terms:
            // stage the plane PC_DEPTH steps ahead into the slot
            __syncwarp();
            if (lane == 0 && s + PC_DEPTH < NP) issue(s + PC_DEPTH, gs + PC_DEPTH);
        }
        if (lane == 0) slot = atomicAdd(w.counter, 1);
        slot = __shfl_sync(0xffffffffu, slot, 0);
    }
    __syncwarp();
    if (lane == 0)
        for (int r = 0; r < PC_DEPTH; r++)
            asm volatile("mbarrier.inval.shared::cta.b64 [%0];" :: "r"(smem_u32(&mbar[warp][r])) : "memory");
}

}  // namespace CF_NS
