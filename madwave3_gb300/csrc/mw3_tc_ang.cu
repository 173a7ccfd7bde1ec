// Angular kinetic terms of the mixed path (difs j^2 + l^2 with the Omega+-1
// Coriolis coupling) as a factorised contraction on the tensor cores.
//
// The reference builds, per block, explicit grid matrices
//   xj2(r1; g, g')    = sum_j Djmmp(g, j) yyy(j, r1)            Djmmp(g', j)   (angkinj2,   SRC/mod_Hphi_01y2.f:166-311)
//   xl2p(R; g, g', q) = sum_j Djmmp(g, j; Om) xl2mat_j(Om, Om+q; R) Djmmp(g', j; Om+q)
//                                                                             (bfgridl2mat, SRC/mod_Hphi_01y2.f:315-484)
// and applies them point by point (SRC/mod_Hphi_01y2.f:856-898).  Both are
// D^T diag D products, so for every (r1, R) point the same result is
//   B_b  = D_b X_b                  grid -> j basis       (GEMM, K = angles)
//   Hb_b = (yyy_b(r1) + l2_b0(R)) B_b + l2_b-(R) B_{b-1} + l2_b+(R) B_{b+1}
//   H_b += D_b^T Hb_b               j basis -> grid       (GEMM, K = j)
// where b-1 / b+1 are the blocks of the same wave and electronic state with
// Omega - 1 / Omega + 1.  A CTA takes one tile of 128 grid points (16 r1 x 8 R)
// and one chain of blocks (one wave, one electronic state, Omega ascending):
// the j-basis coefficients of three consecutive blocks stay in tensor memory
// (ring of three 64-column slots) so the coupling needs no second pass.
//
// Precision: 3xTF32 (hi*hi + hi*lo + lo*hi) with FP32 accumulation, as the
// radial DSTs of the mixed path.  The j-basis operands D_b are split on the
// host into TF32 hi/lo planes in the canonical K-major layout and copied into
// shared memory with one bulk (TMA) copy per GEMM.
#include "mw3_internal.h"
#include "mw3_tc.cuh"

#include <algorithm>
#include <cstring>

namespace mw3 {
namespace tc {

constexpr int AG_K = 64;                          // angles and j-ladder slots, zero padded
constexpr int AG_R1 = 16, AG_R2 = 8;              // tile: 16 r1 x 8 R = 128 rows
constexpr uint32_t AG_APLANE = 128 * AG_K * 4;    // 32 KB: 128 x 64 fp32
constexpr uint32_t AG_DPLANE = 64 * AG_K * 4;     // 16 KB: 64 x 64 fp32
constexpr uint32_t AG_SBO = (AG_K / 4) * 128;     // 2 KB between 8-row groups
constexpr uint32_t AG_BYTES = 2 * AG_APLANE + 2 * AG_DPLANE;   // 96 KB
// the tile's rectangle -> stored-point map (the same for every block) as 16-bit
// indices, [angle][tile row], 0xFFFF = not stored; and the block's flat starts
constexpr uint32_t AG_MAP = AG_K * 128 * 2;       // 16 KB
constexpr uint32_t AG_FO = AG_K * 8;              // 512 B
constexpr uint32_t AG_SMEM = AG_BYTES + AG_MAP + AG_FO + 64;
constexpr uint32_t AG_COLS = 256;                 // three ring slots + the output tile
constexpr uint32_t AG_OUT = 192;                  // column of the output tile

template <typename HT>
struct AngArgs {
    const float *X;              // rectangle [G][na][n1][n2]
    HT *H;                       // flat H accumulator (FP32 when the mixed path keeps H in FP32)
    const float *dfw, *dbk;      // [G][2][64*64] hi/lo planes: (j, angle) and (angle, j), K-major
    const float *yj;             // [G][n1][64]   yyy(j, r1), 0 outside the block's j list
    const float *l2;             // [G][3][n2][64] xl2mat_j(Om, Om+q; R), slot q+1, 0 where absent
    const int *chain_ptr, *chain;
    const int *tiles;            // (r1_0 << 16) | R_0 of the tiles holding stored points
    const int *blk_om, *map;
    const int64_t *foff;
    int na, n1, n2, chain0;
    int xt;                      // rectangle layout: 0 [g][a][r1][R], 1 [g][a][R][r1]
    int *err;
};

// X tile of block g: A operand rows m = (r1 offset)*8 + (R offset), K = angle.
// The tile arrives by asynchronous 4-byte copies straight into the lo plane at
// each element's operand position (zero outside the grid and beyond the angles),
// issued as soon as the operand space is free; later each thread splits its own
// elements into the hi and lo planes in place.  In the [r1][R] layout a quarter
// warp takes 8 consecutive R of one r1 row (one 32-byte sector per angle), in the
// [R][r1] layout a half warp takes the 16 r1 of one R row (64 bytes per angle).
__device__ __forceinline__ void ang_elem(int e, int xt, int &r1o, int &r2o, int &kg)
{
    if (xt) {
        r1o = e & 15;
        r2o = (e >> 4) & 7;
    } else {
        r2o = e & 7;
        r1o = (e >> 3) & 15;
    }
    kg = e >> 7;
}

template <typename HT>
__device__ __forceinline__ void ang_copy_x(const AngArgs<HT> &p, int g, int r1_0, int r2_0, unsigned char *lo)
{
    const float *Xg = p.X + (size_t)g * p.na * p.n1 * p.n2;
    const uint32_t lo_s = smem_u32(lo);
#pragma unroll
    for (int it = 0; it < 8; it++) {
        const int e = threadIdx.x + 256 * it;
        int r1o, r2o, kg;
        ang_elem(e, p.xt, r1o, r2o, kg);
        const int gr1 = r1_0 + r1o, gr2 = r2_0 + r2o;
        const bool in = gr1 < p.n1 && gr2 < p.n2;
        const uint32_t dst = lo_s + kmaj_off(r1o * 8 + r2o, kg * 4, AG_K);
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int a = kg * 4 + c;
            const bool ok = in && a < p.na;
            const size_t at = p.xt ? ((size_t)a * p.n2 + gr2) * p.n1 + gr1 : ((size_t)a * p.n1 + gr1) * p.n2 + gr2;
            const float *src = ok ? Xg + at : Xg;
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst + 4 * c), "l"(src), "r"(ok ? 4 : 0)
                         : "memory");
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// this thread's elements of the copied tile (the same assignment as ang_copy_x):
// wait for its copies, split in place
__device__ __forceinline__ void ang_split_x(unsigned char *hi, unsigned char *lo, int xt)
{
    asm volatile("cp.async.wait_all;" ::: "memory");
#pragma unroll
    for (int it = 0; it < 8; it++) {
        const int e = threadIdx.x + 256 * it;
        int r1o, r2o, kg;
        ang_elem(e, xt, r1o, r2o, kg);
        const int m = r1o * 8 + r2o;
        const uint32_t off = kmaj_off(m, kg * 4, AG_K);
        const float4 x = *reinterpret_cast<const float4 *>(lo + off);
        const float4 h = make_float4(tf32_hi(x.x), tf32_hi(x.y), tf32_hi(x.z), tf32_hi(x.w));
        *reinterpret_cast<float4 *>(hi + off) = h;
        *reinterpret_cast<float4 *>(lo + off) = make_float4(x.x - h.x, x.y - h.y, x.z - h.z, x.w - h.w);
    }
}

// D[128 x 64] (+)= A[128 x 64] B[64 x 64]^T in three TF32 products per K step
__device__ __forceinline__ void ang_issue(uint32_t dcol, const unsigned char *a, const unsigned char *b)
{
    const uint32_t idesc = idesc_tf32(128, 64);
    uint32_t ah = smem_u32(a), al = ah + AG_APLANE, bh = smem_u32(b), bl = bh + AG_DPLANE;
#pragma unroll
    for (int ks = 0; ks < AG_K / 8; ks++) {
        uint32_t o = ks * 256;
        uint64_t dah = sdesc(ah + o, 128, AG_SBO), dal = sdesc(al + o, 128, AG_SBO);
        uint64_t dbh = sdesc(bh + o, 128, AG_SBO), dbl = sdesc(bl + o, 128, AG_SBO);
        mma_tf32(dcol, dah, dbh, idesc, ks > 0 ? 1 : 0);
        mma_tf32(dcol, dah, dbl, idesc, 1);
        mma_tf32(dcol, dal, dbh, idesc, 1);
    }
}

template <typename HT>
__global__ void __launch_bounds__(256, 2) k_tc_ang(AngArgs<HT> p)
{
    // the no-swizzle operand layout needs 16-byte alignment only; keeping the
    // footprint at 113 KB lets two CTAs share an SM
    extern __shared__ __align__(128) unsigned char smraw[];
    unsigned char *sm = smraw;
    unsigned char *AS = sm;                            // A operand: X tile, then Hb
    unsigned char *DS = sm + 2 * AG_APLANE;            // B operand: D_fw, then D_bk
    uint16_t *s_map = reinterpret_cast<uint16_t *>(sm + AG_BYTES);
    int64_t *s_fo = reinterpret_cast<int64_t *>(sm + AG_BYTES + AG_MAP);
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + AG_BYTES + AG_MAP + AG_FO);   // [0] bulk copy, [1] MMA
    uint32_t *slot = reinterpret_cast<uint32_t *>(bars + 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) tmem_alloc(slot, AG_COLS);
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tb = *slot;
    const int na = p.na, n1 = p.n1, n2 = p.n2;
    const int tile = p.tiles[blockIdx.x];
    const int r1_0 = tile >> 16, r2_0 = tile & 0xFFFF;
    const int ch = p.chain0 + blockIdx.y;
    const int cb = p.chain_ptr[ch], L = p.chain_ptr[ch + 1] - cb;
    // the tile's map, once for the whole chain (a quarter warp reads 8 consecutive R)
    for (int e = threadIdx.x; e < AG_K * 128; e += blockDim.x) {
        int a = e >> 7, mm = e & 127;
        int gr1 = r1_0 + (mm >> 3), gr2 = r2_0 + (mm & 7);
        int v = (a < na && gr1 < n1 && gr2 < n2) ? __ldg(p.map + ((size_t)a * n1 + gr1) * n2 + gr2) : -1;
        s_map[e] = v < 0 ? (uint16_t)0xFFFF : (uint16_t)v;
    }
    // this thread's tile row (tensor-memory lane) and column half
    const int q4 = warp & 3, half = warp >> 2;
    const int m = q4 * 32 + lane;
    const int ir1 = r1_0 + (m >> 3), ir2 = r2_0 + (m & 7);
    const int cr1 = min(ir1, n1 - 1), cr2 = min(ir2, n2 - 1);
    const uint32_t lrow = tb + ((uint32_t)(q4 * 32) << 16);
    uint32_t ph0 = 0, ph1 = 0;
    bool bad = false, copy_out = false;
    if (L > 0) ang_copy_x(p, p.chain[cb], r1_0, r2_0, AS + AG_APLANE);

    for (int pos = -1; pos < L; pos++) {
        // the X tile of the block after next into L2 (one 32-byte run per angle and r1
        // row), and this block's j-basis rows into L1 for the scaling below
        if (pos + 2 < L) {
            const float *Xn = p.X + (size_t)p.chain[cb + pos + 2] * na * n1 * n2;
            if (p.xt) {
                for (int e = threadIdx.x; e < na * AG_R2; e += blockDim.x) {
                    int a = e >> 3, gr2 = r2_0 + (e & 7);
                    if (gr2 < n2) asm volatile("prefetch.global.L2 [%0];" ::"l"(Xn + ((size_t)a * n2 + gr2) * n1 + r1_0));
                }
            } else {
                for (int e = threadIdx.x; e < na * AG_R1; e += blockDim.x) {
                    int a = e >> 4, gr1 = r1_0 + (e & 15);
                    if (gr1 < n1)
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(Xn + ((size_t)a * n1 + gr1) * n2 + r2_0));
                }
            }
        }
        if (pos >= 0) {
            const int g = p.chain[cb + pos];
            const float *yrow = p.yj + ((size_t)g * n1 + cr1) * AG_K;
            const float *lr = p.l2 + ((size_t)g * 3 * n2 + cr2) * AG_K;
            const size_t lslot = (size_t)n2 * AG_K;
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                asm volatile("prefetch.global.L1 [%0];" ::"l"(yrow + 32 * hh));
#pragma unroll
                for (int q = 0; q < 3; q++) asm volatile("prefetch.global.L1 [%0];" ::"l"(lr + q * lslot + 32 * hh));
            }
        }
        // ---- grid -> j basis for the next block of the chain, into ring slot (pos+1)%3 ----
        if (pos + 1 < L) {
            int gn = p.chain[cb + pos + 1];
            if (threadIdx.x == 0) {
                mbar_expect_tx(&bars[0], 2 * AG_DPLANE);
                bulk_g2s(DS, p.dfw + (size_t)gn * 2 * 64 * AG_K, 2 * AG_DPLANE, &bars[0]);
                copy_out = true;
            }
            ang_split_x(AS, AS + AG_APLANE, p.xt);
            fence_async_smem();
            fence_before_sync();
            if (__syncthreads_or(bad)) break;
            if (threadIdx.x == 0) {
                if (!mbar_wait(&bars[0], ph0)) bad = true;
                copy_out = false;
                fence_after_sync();
                if (!bad) ang_issue(tb + ((pos + 1) % 3) * 64, AS, DS);
                mma_commit(&bars[1]);
            }
            ph0 ^= 1u;
            if (!mbar_wait(&bars[1], ph1)) bad = true;
            ph1 ^= 1u;
            fence_after_sync();
        }
        if (pos < 0) {
            // the first block's tile has been read: the second block's tile can come in
            if (!__syncthreads_or(bad) && L > 1) ang_copy_x(p, p.chain[cb + 1], r1_0, r2_0, AS + AG_APLANE);
            continue;
        }
        if (__syncthreads_or(bad)) break;
        // ---- scaling and coupling in the j basis ----
        const int g = p.chain[cb + pos];
        const int om = p.blk_om[g];
        const bool hp = pos > 0 && p.blk_om[p.chain[cb + pos - 1]] == om - 1;
        const bool hn = pos + 1 < L && p.blk_om[p.chain[cb + pos + 1]] == om + 1;
        // the block's flat starts for the epilogue (every thread is past the previous
        // epilogue here; the barrier after Hb publishes them)
        if (threadIdx.x < na) s_fo[threadIdx.x] = __ldg(p.foff + (size_t)g * na + threadIdx.x);
        if (threadIdx.x == 0) {              // D_b^T for the way back, while Hb is formed
            mbar_expect_tx(&bars[0], 2 * AG_DPLANE);
            bulk_g2s(DS, p.dbk + (size_t)g * 2 * 64 * AG_K, 2 * AG_DPLANE, &bars[0]);
            copy_out = true;
        }
        {
            const uint32_t s0 = lrow + (pos % 3) * 64, sp = lrow + ((pos + 2) % 3) * 64,
                           sn = lrow + ((pos + 1) % 3) * 64;
            const float *yrow = p.yj + ((size_t)g * n1 + cr1) * AG_K;
            const float *lrow0 = p.l2 + ((size_t)g * 3 * n2 + cr2) * AG_K;
            const size_t lslot = (size_t)n2 * AG_K;
            // The scale rows are shared: the 32 lanes of a warp cover 4 r1 rows (lane >> 3)
            // and 8 R rows (lane & 7).  Each lane loads a slice of its rows (two yyy
            // values, four of each xl2mat slot) and the values are passed between lanes,
            // instead of every lane loading all of its own rows.
            const int gq = lane >> 3, rq = lane & 7;
#pragma unroll
            for (int cc = 0; cc < 2; cc++) {
                const int j0 = half * 32 + cc * 16;
                const float2 ys = *reinterpret_cast<const float2 *>(yrow + j0 + 2 * rq);
                const float4 l0s = *reinterpret_cast<const float4 *>(lrow0 + lslot + j0 + 4 * gq);
                const float4 lms = hp ? *reinterpret_cast<const float4 *>(lrow0 + j0 + 4 * gq)
                                      : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 lqs = hn ? *reinterpret_cast<const float4 *>(lrow0 + 2 * lslot + j0 + 4 * gq)
                                      : make_float4(0.f, 0.f, 0.f, 0.f);
                float b0[16], bp[16], bn[16];
                tmem_ld16(s0 + j0, b0);
                if (hp) tmem_ld16(sp + j0, bp);
                if (hn) tmem_ld16(sn + j0, bn);
#pragma unroll
                for (int i4 = 0; i4 < 4; i4++) {
                    const int j = j0 + 4 * i4;
                    float hb[4];
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        // yyy(j0 + 4 i4 + e) of this lane's r1 row, xl2mat of its R row
                        const float y = __shfl_sync(0xffffffffu, (e & 1) ? ys.y : ys.x, (lane & 24) + 2 * i4 + (e >> 1));
                        const int src = 8 * i4 + rq;
                        const float l0 = __shfl_sync(0xffffffffu, e == 0 ? l0s.x : e == 1 ? l0s.y : e == 2 ? l0s.z : l0s.w, src);
                        hb[e] = (y + l0) * b0[4 * i4 + e];
                        if (hp) {
                            const float lm = __shfl_sync(0xffffffffu, e == 0 ? lms.x : e == 1 ? lms.y : e == 2 ? lms.z : lms.w, src);
                            hb[e] += lm * bp[4 * i4 + e];
                        }
                        if (hn) {
                            const float lq = __shfl_sync(0xffffffffu, e == 0 ? lqs.x : e == 1 ? lqs.y : e == 2 ? lqs.z : lqs.w, src);
                            hb[e] += lq * bn[4 * i4 + e];
                        }
                    }
                    float4 h = make_float4(tf32_hi(hb[0]), tf32_hi(hb[1]), tf32_hi(hb[2]), tf32_hi(hb[3]));
                    float4 l = make_float4(hb[0] - h.x, hb[1] - h.y, hb[2] - h.z, hb[3] - h.w);
                    uint32_t off = kmaj_off(m, j, AG_K);
                    *reinterpret_cast<float4 *>(AS + off) = h;
                    *reinterpret_cast<float4 *>(AS + AG_APLANE + off) = l;
                }
            }
        }
        fence_async_smem();
        fence_before_sync();
        if (__syncthreads_or(bad)) break;
        // ---- j basis -> grid ----
        if (threadIdx.x == 0) {
            if (!mbar_wait(&bars[0], ph0)) bad = true;
            copy_out = false;
            fence_after_sync();
            if (!bad) ang_issue(tb + AG_OUT, AS, DS);
            mma_commit(&bars[1]);
        }
        ph0 ^= 1u;
        if (!mbar_wait(&bars[1], ph1)) bad = true;
        ph1 ^= 1u;
        fence_after_sync();
        if (__syncthreads_or(bad)) break;
        // the operand space is free again: the X tile of the block after next starts
        // arriving while this block's H is written
        if (pos + 2 < L) ang_copy_x(p, p.chain[cb + pos + 2], r1_0, r2_0, AS + AG_APLANE);
        // ---- H += result at the stored points of this block ----
        {
#pragma unroll
            for (int cc = 0; cc < 2; cc++) {
                const int a0 = half * 32 + cc * 16;
                float v[16];
                tmem_ld16(lrow + AG_OUT + a0, v);
#pragma unroll
                for (int h8 = 0; h8 < 16; h8 += 8) {
                    int64_t at[8];
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        int a = a0 + h8 + i;
                        unsigned idx = s_map[a * 128 + m];
                        at[i] = (a < na && idx != 0xFFFFu) ? s_fo[a] + (int64_t)idx : -1;
                    }
                    // one writer per point in this launch: a fire-and-forget add at L2
                    // instead of a load and a store (no load latency in the epilogue)
#pragma unroll
                    for (int i = 0; i < 8; i++)
                        if (at[i] >= 0) atomicAdd(p.H + at[i], (HT)v[h8 + i]);
                }
            }
        }
        fence_before_sync();
    }
    if (bad && threadIdx.x == 0) atomicExch(p.err, 1);
    // copies of an X tile still in flight (after a failure) land before the CTA exits
    asm volatile("cp.async.wait_all;" ::: "memory");
    // a bulk copy left in flight by a failed wait must land before the CTA exits
    if (copy_out) mbar_wait(&bars[0], ph0);
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tb, AG_COLS);
}

}  // namespace tc

namespace {

float tf32_round_host(float x)
{
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;      // nearest, ties away from zero, on the magnitude bits
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

// float index of (r, k) in a canonical K-major plane with K extent 64
inline size_t kmaj_idx(int r, int k)
{
    return (size_t)(((r & 7) * 16 + (r >> 3) * (tc::AG_K / 4) * 128 + (k & 3) * 4 + (k >> 2) * 128) / 4);
}

template <typename V>
int upload(Ctx &c, V **dst, const std::vector<V> &v)
{
    *dst = nullptr;
    size_t bytes = sizeof(V) * std::max<size_t>(v.size(), 1);
    cudaError_t e = cudaMalloc((void **)dst, bytes);
    if (e != cudaSuccess) {
        c.err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return MW3_ERR_CUDA;
    }
    c.allocs.push_back(*dst);
    if (!v.empty()) {
        e = cudaMemcpy(*dst, v.data(), sizeof(V) * v.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            c.err = std::string("cudaMemcpy: ") + cudaGetErrorString(e);
            return MW3_ERR_CUDA;
        }
    }
    return MW3_OK;
}

}  // namespace

// Tables of the factorised angular contraction.  Returns MW3_OK with
// c.use_tc_ang = false when the shape is outside what the kernel covers
// (more than 64 angles or j values, a block whose j list leaves the ladder
// j0 + k*inc, or Omega couplings that are not chain neighbours); the explicit
// kernels then stay in use.
int build_tc_ang(Ctx &c)
{
    using tc::AG_K;
    c.use_tc_ang = false;
    if (c.fp64 || !c.use_tc || c.k_ang == 0 || c.na < 2 || c.na > AG_K) return MW3_OK;
    if (c.npt >= 0xFFFF) return MW3_OK;                // the tile map holds 16-bit point indices
    const int na = c.na, n1 = c.n1, n2 = c.n2, G = c.G;
    std::vector<float> dfw((size_t)G * 2 * 64 * AG_K, 0.f), dbk((size_t)G * 2 * 64 * AG_K, 0.f);
    std::vector<float> yj((size_t)G * n1 * AG_K, 0.f), l2((size_t)G * 3 * n2 * AG_K, 0.f);
    std::vector<int> chain_ptr(1, 0), chain;
    c.ang_wchain.assign(c.waves.size() + 1, 0);
    for (size_t w = 0; w < c.waves.size(); w++) {
        const WaveTables &t = c.waves[w];
        int njl = 0;                                   // ladder j = j0 + k*inc <= (na-1)*inc and <= nangu2
        while (njl < t.nj2 && t.j0 + njl * t.inc <= (na - 1) * t.inc && t.j0 + njl * t.inc <= t.nangu2) njl++;
        if (njl > AG_K) return MW3_OK;
        for (int b = 0; b < t.ncan; b++) {
            int g = t.g0 + b, om = t.iombas[b], e = t.nelebas[b];
            // Djmmp(angle, j; e, Om) in both operand layouts, split into hi/lo
            for (int js = 0; js < njl; js++) {
                int jv = t.j0 + js * t.inc;
                for (int a = 0; a < na; a++) {
                    double d = t.djmmp[(((size_t)om * c.ne + (e - 1)) * (t.nangu2 + 1) + jv) * na + a];
                    float x = (float)d, h = tf32_round_host(x), l = x - h;
                    size_t fw = kmaj_idx(js, a), bk = kmaj_idx(a, js);
                    size_t base = (size_t)g * 2 * 64 * AG_K;
                    dfw[base + fw] = h;
                    dfw[base + 64 * AG_K + fw] = l;
                    dbk[base + bk] = h;
                    dbk[base + 64 * AG_K + bk] = l;
                }
            }
            // yyy of the block's own j list, by ladder slot
            for (int k = 0; k < t.nojbas[b]; k++) {
                int jb = t.jbas[(size_t)b * na + k];
                bool any = false;
                for (int ir1 = 0; ir1 < n1; ir1++) any |= t.yj2[((size_t)b * n1 + ir1) * na + k] != 0.0;
                if (!any) continue;
                if ((jb - t.j0) % t.inc != 0 || (jb - t.j0) / t.inc < 0 || (jb - t.j0) / t.inc >= njl)
                    return MW3_OK;
                int js = (jb - t.j0) / t.inc;
                for (int ir1 = 0; ir1 < n1; ir1++)
                    yj[((size_t)g * n1 + ir1) * AG_K + js] += (float)t.yj2[((size_t)b * n1 + ir1) * na + k];
            }
            // xl2mat_j(Om, Om+q; R) for the sources Om+q, q = -1, 0, +1
            for (int q = -1; q <= 1; q++) {
                int oms = om + q;
                if (oms < t.iommin || oms > t.iommax) continue;
                // the source must be the chain neighbour (or the block itself)
                int src = -1;
                for (int s = 0; s < t.ncan; s++)
                    if (t.nelebas[s] == e && t.iombas[s] == oms) src = s;
                for (int js = 0; js < std::min(njl, t.nj2); js++) {
                    size_t u = (((size_t)(e - 1) * t.nj2 + js) * t.nom + (om - t.iommin)) * t.nom + (oms - t.iommin);
                    if (!t.l2used[u] || src < 0) continue;
                    for (int ir2 = 0; ir2 < n2; ir2++) {
                        double y = t.l2tab[((((size_t)(e - 1) * t.nj2 + js) * n2 + ir2) * t.nom + (om - t.iommin)) *
                                               t.nom + (oms - t.iommin)];
                        l2[(((size_t)g * 3 + (q + 1)) * n2 + ir2) * AG_K + js] = (float)y;
                    }
                }
            }
        }
        // chains: one per electronic state, blocks by ascending Omega
        for (int e = 1; e <= c.ne; e++) {
            std::vector<std::pair<int, int>> bl;
            for (int b = 0; b < t.ncan; b++)
                if (t.nelebas[b] == e) bl.push_back({t.iombas[b], t.g0 + b});
            if (bl.empty()) continue;
            std::sort(bl.begin(), bl.end());
            for (size_t i = 1; i < bl.size(); i++)
                if (bl[i].first == bl[i - 1].first) return MW3_OK;     // two blocks with one Omega
            for (auto &x : bl) chain.push_back(x.second);
            chain_ptr.push_back((int)chain.size());
        }
        c.ang_wchain[w + 1] = (int)chain_ptr.size() - 1;
    }
    // tiles of 16 r1 x 8 R holding at least one stored point
    int t1n = (n1 + tc::AG_R1 - 1) / tc::AG_R1, t2n = (n2 + tc::AG_R2 - 1) / tc::AG_R2;
    std::vector<char> on((size_t)t1n * t2n, 0);
    for (int a = 0; a < na; a++)
        for (int ir = 0; ir < c.npunreal[a]; ir++) {
            int ir1 = c.indr1[(size_t)a * c.npt + ir] - 1, ir2 = c.indr2[(size_t)a * c.npt + ir] - 1;
            on[(size_t)(ir1 / tc::AG_R1) * t2n + ir2 / tc::AG_R2] = 1;
        }
    std::vector<int> tiles;
    for (int i = 0; i < t1n; i++)
        for (int j = 0; j < t2n; j++)
            if (on[(size_t)i * t2n + j]) tiles.push_back(((i * tc::AG_R1) << 16) | (j * tc::AG_R2));
    if (tiles.empty() || n2 > 0xFFFF) return MW3_OK;
    int rc;
    if ((rc = upload(c, &c.d_ang_dfw, dfw))) return rc;
    if ((rc = upload(c, &c.d_ang_dbk, dbk))) return rc;
    if ((rc = upload(c, &c.d_ang_yj, yj))) return rc;
    if ((rc = upload(c, &c.d_ang_l2, l2))) return rc;
    if ((rc = upload(c, &c.d_ang_chain_ptr, chain_ptr))) return rc;
    if ((rc = upload(c, &c.d_ang_chain, chain))) return rc;
    if ((rc = upload(c, &c.d_ang_tiles, tiles))) return rc;
    c.ang_ntiles = (int)tiles.size();
    c.use_tc_ang = true;
    return MW3_OK;
}

// blocks [g_begin, g_end) must be whole waves
template <typename HT>
static void tc_ang_launch(Ctx &c, const float *X, HT *H, int g_begin, int g_end, bool xt)
{
    using namespace tc;
    static bool attr = false;
    const size_t smem = AG_SMEM;
    if (!attr) {
        cudaFuncSetAttribute(k_tc_ang<HT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    int w0 = c.waves.size(), w1 = 0;
    for (size_t w = 0; w < c.waves.size(); w++) {
        const WaveTables &t = c.waves[w];
        if (t.g0 >= g_begin && t.g0 + t.ncan <= g_end) {
            w0 = std::min(w0, (int)w);
            w1 = std::max(w1, (int)w + 1);
        }
    }
    if (w1 <= w0) return;
    int ch0 = c.ang_wchain[w0], nch = c.ang_wchain[w1] - ch0;
    if (nch <= 0) return;
    AngArgs<HT> p;
    p.X = X; p.H = H;
    p.dfw = c.d_ang_dfw; p.dbk = c.d_ang_dbk; p.yj = c.d_ang_yj; p.l2 = c.d_ang_l2;
    p.chain_ptr = c.d_ang_chain_ptr; p.chain = c.d_ang_chain; p.tiles = c.d_ang_tiles;
    p.blk_om = c.d_blk_om; p.map = c.d_map; p.foff = c.d_foff;
    p.na = c.na; p.n1 = c.n1; p.n2 = c.n2; p.chain0 = ch0;
    p.xt = xt ? 1 : 0;
    p.err = c.d_tc_err;
    k_tc_ang<HT><<<dim3(c.ang_ntiles, nch), 256, smem, c.stream>>>(p);
    c.launches++;
}

void launch_tc_ang(Ctx &c, const float *X, double *H, int g_begin, int g_end, bool xt)
{
    tc_ang_launch<double>(c, X, H, g_begin, g_end, xt);
}

void launch_tc_ang(Ctx &c, const float *X, float *H, int g_begin, int g_end, bool xt)
{
    tc_ang_launch<float>(c, X, H, g_begin, g_end, xt);
}

}  // namespace mw3
