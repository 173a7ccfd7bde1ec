// Tensor-core (tcgen05, kind::tf32, 3xTF32 split) GEMM tile used by the mixed
// path's radial DSTs, plus a self-test entry point for the test suite.
//
// One CTA computes a 128 x BN tile of C = A * Bt^T (A: M x K, Bt: N x K, both
// row-major FP32).  K streams through two shared-memory stages of KC = 32
// columns; one thread issues the MMAs (three per K step of 8: hi*hi, hi*lo,
// lo*hi) and commits each stage to an mbarrier that gates its reuse.  The
// accumulator lives in tensor memory (BN columns x 128 lanes) and is read back
// with tcgen05.ld by the four warps, one 32-lane quarter each.
#include "mw3_internal.h"
#include "mw3_tc.cuh"

namespace mw3 {
namespace tc {

constexpr int KC = 32;                        // K columns per stage
constexpr uint32_t A_PLANE = 128 * KC * 4;    // 16 KB: one 128 x KC fp32 plane
constexpr uint32_t SBO = (KC / 4) * 128;      // 1 KB between 8-row groups

template <int BN>
struct TileSmem {
    static constexpr uint32_t B_PLANE = BN * KC * 4;
    static constexpr uint32_t STAGE = 2 * A_PLANE + 2 * B_PLANE;
    static constexpr uint32_t BYTES = 2 * STAGE + 1024;   // two stages + barriers/slot
};

// Staging of a row tile [r0, r0+NR) x [k0, k0+KC) of a row-major matrix into
// hi/lo planes, in two halves so the global loads of the next K chunk can be in
// flight while the tensor cores work on the current one.  Thread mapping: the 8
// lanes of a quarter warp take rows r..r+7 of one 16-byte column group, so every
// quarter-warp store is one contiguous 128-byte core-matrix block.
template <int NR>
struct RowStage {
    static constexpr int PER = NR * (KC / 4) / 128;    // float4 per thread (128 threads)
    float4 v[PER];
    __device__ __forceinline__ static void idx(int e, int &r, int &kg)
    {
        int rest = e >> 3;
        kg = rest % (KC / 4);
        r = (rest / (KC / 4)) * 8 + (e & 7);
    }
    __device__ __forceinline__ void load(const float *src, int64_t ld, int64_t rows, int cols, int64_t r0, int k0)
    {
#pragma unroll
        for (int i = 0; i < PER; i++) {
            int r, kg;
            idx(threadIdx.x + 128 * i, r, kg);
            int64_t gr = r0 + r;
            int gk = k0 + kg * 4;
            float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
            if (gr < rows) {
                const float *p = src + gr * ld + gk;
                if (gk + 3 < cols && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
                    x = __ldg(reinterpret_cast<const float4 *>(p));
                } else {
                    if (gk < cols) x.x = p[0];
                    if (gk + 1 < cols) x.y = p[1];
                    if (gk + 2 < cols) x.z = p[2];
                    if (gk + 3 < cols) x.w = p[3];
                }
            }
            v[i] = x;
        }
    }
    __device__ __forceinline__ void store(unsigned char *hi, unsigned char *lo) const
    {
#pragma unroll
        for (int i = 0; i < PER; i++) {
            int r, kg;
            idx(threadIdx.x + 128 * i, r, kg);
            float4 h = make_float4(tf32_hi(v[i].x), tf32_hi(v[i].y), tf32_hi(v[i].z), tf32_hi(v[i].w));
            float4 l = make_float4(v[i].x - h.x, v[i].y - h.y, v[i].z - h.z, v[i].w - h.w);
            uint32_t off = kmaj_off(r, kg * 4, KC);
            *reinterpret_cast<float4 *>(hi + off) = h;
            *reinterpret_cast<float4 *>(lo + off) = l;
        }
    }
};

// single-shot staging (loads and stores back to back)
__device__ __forceinline__ void stage_rows(unsigned char *hi, unsigned char *lo, const float *src, int64_t ld,
                                           int64_t rows, int cols, int64_t r0, int nr, int k0)
{
    if (nr == 128) {
        RowStage<128> st;
        st.load(src, ld, rows, cols, r0, k0);
        st.store(hi, lo);
    } else {
        RowStage<256> st;
        st.load(src, ld, rows, cols, r0, k0);
        st.store(hi, lo);
    }
}

// C tile = A[row0:row0+128, :K] * Bt[col0:col0+BN, :K]^T, accumulated in tensor
// memory; returns false when an mbarrier wait ran out (error reported by the caller).
template <int BN>
__device__ bool tile_mma(unsigned char *sm, const float *A, int64_t lda, int64_t M, const float *Bt, int64_t ldb,
                         int64_t N, int K, int64_t row0, int64_t col0, uint32_t taddr, uint64_t *bars)
{
    constexpr uint32_t STAGE = TileSmem<BN>::STAGE, B_PLANE = TileSmem<BN>::B_PLANE;
    const uint32_t idesc = idesc_tf32(128, BN);
    int nk = (K + KC - 1) / KC;
    uint32_t phase[2] = {0u, 0u};
    bool ok = true;
    RowStage<128> sa;
    RowStage<BN> sb;
    sa.load(A, lda, M, K, row0, 0);
    sb.load(Bt, ldb, N, K, col0, 0);
    for (int kc = 0; kc < nk; kc++) {
        int s = kc & 1;
        unsigned char *st = sm + s * STAGE;
        if (kc >= 2) {
            if (!mbar_wait(&bars[s], phase[s])) ok = false;
            phase[s] ^= 1u;
        }
        sa.store(st, st + A_PLANE);
        sb.store(st + 2 * A_PLANE, st + 2 * A_PLANE + B_PLANE);
        if (kc + 1 < nk) {                       // next chunk's loads overlap this chunk's MMAs
            sa.load(A, lda, M, K, row0, (kc + 1) * KC);
            sb.load(Bt, ldb, N, K, col0, (kc + 1) * KC);
        }
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0 && ok) {
            fence_after_sync();
            uint32_t ah = smem_u32(st), al = ah + A_PLANE, bh = ah + 2 * A_PLANE, bl = bh + B_PLANE;
#pragma unroll
            for (int ks = 0; ks < KC / 8; ks++) {
                uint32_t o = ks * 256;
                uint64_t dah = sdesc(ah + o, 128, SBO), dal = sdesc(al + o, 128, SBO);
                uint64_t dbh = sdesc(bh + o, 128, SBO), dbl = sdesc(bl + o, 128, SBO);
                mma_tf32(taddr, dah, dbh, idesc, (kc > 0 || ks > 0) ? 1 : 0);
                mma_tf32(taddr, dah, dbl, idesc, 1);
                mma_tf32(taddr, dal, dbh, idesc, 1);
            }
            mma_commit(&bars[s]);
        }
    }
    // the last commit tracks every MMA issued before it
    int last = (nk - 1) & 1;
    if (!mbar_wait(&bars[last], phase[last])) ok = false;
    fence_after_sync();
    return ok;
}

// Tensor-memory tile -> shared memory [128][BN] (row stride BN, 32-float blocks
// XOR-swizzled by row so both the row writes here and the column reads later
// are free of bank conflicts).  Must be called by all 128 threads.
template <int BN>
__device__ __forceinline__ void tmem_to_smem(uint32_t taddr, float *tile)
{
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int m = warp * 32 + lane;
    for (int cc = 0; cc < BN / 32; cc++) {
        float v[32];
        tmem_ld32(taddr + ((uint32_t)(warp * 32) << 16) + cc * 32, v);
#pragma unroll
        for (int i = 0; i < 32; i++) tile[(size_t)m * BN + cc * 32 + (i ^ lane)] = v[i];
    }
}

__device__ __forceinline__ float tile_get(const float *tile, int bn, int m, int n)
{
    return tile[(size_t)m * bn + (n & ~31) + ((n & 31) ^ (m & 31))];
}

template <int BN>
__global__ void __launch_bounds__(128) k_tc_gemm_test(const float *A, const float *Bt, float *C, int M, int N, int K,
                                                     int *err)
{
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char *sm = smraw + ((1024 - (smem_u32(smraw) & 1023)) & 1023);
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + 2 * TileSmem<BN>::STAGE);
    uint32_t *slot = reinterpret_cast<uint32_t *>(bars + 2);
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) tmem_alloc(slot, BN);
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    uint32_t taddr = *slot;
    int64_t row0 = (int64_t)blockIdx.y * 128, col0 = (int64_t)blockIdx.x * BN;
    bool ok = tile_mma<BN>(sm, A, K, M, Bt, K, N, K, row0, col0, taddr, bars);
    if (!ok && lane == 0) atomicExch(err, 1);
    int64_t r = row0 + warp * 32 + lane;
    for (int cc = 0; cc < BN / 32; cc++) {
        float v[32];
        tmem_ld32(taddr + ((uint32_t)(warp * 32) << 16) + cc * 32, v);
        if (r < M)
            for (int i = 0; i < 32; i++) {
                int64_t col = col0 + cc * 32 + i;
                if (col < N) C[r * N + col] = v[i];
            }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(taddr, BN);
}

// ---------------------------------------------------------------------------
// radial DSTs of the mixed path (difs T-part, SRC/mod_Hphi_01y2.f:752-832)
// ---------------------------------------------------------------------------

__device__ __forceinline__ void setup_cta(unsigned char *sm, uint32_t stage_bytes, int nbars, uint32_t ncols,
                                          uint64_t **bars, uint32_t *taddr)
{
    *bars = reinterpret_cast<uint64_t *>(sm + stage_bytes);
    uint32_t *slot = reinterpret_cast<uint32_t *>(*bars + nbars);
    if ((threadIdx.x >> 5) == 0) tmem_alloc(slot, ncols);
    if (threadIdx.x == 0) {
        for (int i = 0; i < nbars; i++) mbar_init(&(*bars)[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    *taddr = *slot;
}

__device__ __forceinline__ void teardown_cta(uint32_t taddr, uint32_t ncols)
{
    fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tmem_dealloc(taddr, ncols);
}

// R direction: C[r][:] = A[r][:] S2 for the rows r = (block, angle, ir1) of the
// rectangle with ir1 < nopr1; GATHER writes the result at the stored points into H.
template <bool GATHER>
__global__ void __launch_bounds__(128) k_tc_dst_rows(DevGrid d, const float *__restrict__ A, const float *__restrict__ S,
                                                    float *__restrict__ C, double *__restrict__ H,
                                                    const int *__restrict__ nopr1, int64_t row0, int64_t nrows,
                                                    int *__restrict__ err)
{
    constexpr int BN = 128;
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char *sm = smraw + ((1024 - (smem_u32(smraw) & 1023)) & 1023);
    const int n1 = d.n1, n2 = d.n2, na = d.na;
    int64_t rbase = row0 + (int64_t)blockIdx.x * 128, col0 = (int64_t)blockIdx.y * BN;
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    {
        int64_t r = rbase + threadIdx.x;
        if (r < row0 + nrows) {
            int64_t ga = r / n1;
            int ir1 = (int)(r % n1);
            int g = (int)(ga / na), a = (int)(ga % na);
            if (ir1 < nopr1[d.blk_wave[g] * na + a]) any = 1;
        }
    }
    __syncthreads();
    if (!any) return;
    uint64_t *bars;
    uint32_t taddr;
    setup_cta(sm, 2 * TileSmem<BN>::STAGE, 2, BN, &bars, &taddr);
    bool ok = tile_mma<BN>(sm, A, n2, row0 + nrows, S, n2, n2, n2, rbase, col0, taddr, bars);
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    // stage the tile through the (now idle) operand buffers, then write it out
    float *tile = reinterpret_cast<float *>(sm);                       // stage 0: 64 KB
    int *mtile = reinterpret_cast<int *>(sm + TileSmem<BN>::STAGE);     // stage 1: map tile [BN][128]
    __shared__ int r_ir1[128], r_a[128], r_on[128];
    __shared__ long long r_foff[128];
    {
        int m = threadIdx.x;
        int64_t r = rbase + m;
        int on = 0, ga = 0, ir1 = 0, a = 0;
        if (r < row0 + nrows) {
            int rr = (int)r;                       // row counts fit 32 bits
            ga = rr / n1;
            ir1 = rr - ga * n1;
            a = ga % na;
            on = ir1 < nopr1[d.blk_wave[ga / na] * na + a];
        }
        r_ir1[m] = ir1; r_a[m] = a; r_on[m] = on;
        r_foff[m] = GATHER && on ? (long long)d.foff[ga] : 0;
    }
    __syncthreads();
    if (GATHER) {
        // the tile's rectangle->stored-point map, loaded with every thread's
        // loads in flight at once (rows of one tile may belong to two angles)
        constexpr int U = 8;                      // loads in flight per thread
        for (int e0 = threadIdx.x; e0 < BN * 128; e0 += U * 128) {
            int v[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                int e = e0 + u * 128, n = e >> 7, m = e & 127;
                int col = (int)col0 + n;
                v[u] = (e < BN * 128 && r_on[m] && col < n2)
                           ? __ldg(d.mapT + ((size_t)r_a[m] * n2 + col) * n1 + r_ir1[m])
                           : -1;
            }
#pragma unroll
            for (int u = 0; u < U; u++)
                if (e0 + u * 128 < BN * 128) mtile[e0 + u * 128] = v[u];
        }
    }
    tmem_to_smem<BN>(taddr, tile);
    __syncthreads();
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (GATHER) {
        // R points per warp, r1 points across lanes: stored points of one R value
        // are consecutive in r1, so the H writes coalesce
        for (int n = warp; n < BN; n += 4) {
#pragma unroll
            for (int t = 0; t < 4; t++) {
                int m = t * 32 + lane;
                int idx = mtile[n * 128 + m];
                if (idx >= 0) H[r_foff[m] + idx] = (double)tile_get(tile, BN, m, n);
            }
        }
    } else {
        for (int m = warp; m < 128; m += 4) {
            if (!r_on[m]) continue;
            float *cr = C + (rbase + m) * n2 + col0;
            for (int n = lane; n < BN; n += 32)
                if (col0 + n < n2) cr[n] = tile_get(tile, BN, m, n);
        }
    }
    teardown_cta(taddr, BN);
}

// r direction for one (block, angle) and 128 columns, both DSTs of the pair with
// the k-space scaling between them kept on chip:
//   U = S1 Y[0:nn, cols];  U <- U o min(p2r1 + p2r2, radcut) / (4(nn+1)(n2+1));  Y[0:nn, cols] = S1 U
// nn = nopr1 <= 128.  Shared memory: two A stages (S1 chunks) then a region
// that first holds the two Y stages and then the whole scaled U as B operand.
constexpr int COLS_BN = 128;
constexpr uint32_t COLS_B1_STAGE = 2 * (COLS_BN * KC * 4);        // hi + lo, 32 KB
constexpr uint32_t COLS_B2 = 2 * (COLS_BN * 128 * 4);             // hi + lo, 128 KB
constexpr uint32_t COLS_A_OFF = 0;                                 // 2 x 32 KB
constexpr uint32_t COLS_B_OFF = 2 * 2 * A_PLANE;                   // 64 KB
constexpr uint32_t COLS_BYTES = COLS_B_OFF + COLS_B2;              // 192 KB (+ barriers)

// Transposed staging of Y[k0:k0+KC][col0:col0+128] as the K-major operand
// Bt[n][k]: thread n loads four k per column group (coalesced along n) and
// stores one float4 per group; a quarter warp covers one 128-byte block.
struct ColStage {
    float v[KC];
    __device__ __forceinline__ void load(const float *Y, int n2, int nn, int k0, int col0)
    {
        int n = threadIdx.x, gc = col0 + n;
#pragma unroll
        for (int k = 0; k < KC; k++) {
            int gk = k0 + k;
            v[k] = (gk < nn && gc < n2) ? __ldg(Y + (size_t)gk * n2 + gc) : 0.f;
        }
    }
    __device__ __forceinline__ void store(unsigned char *hi, unsigned char *lo) const
    {
        int n = threadIdx.x;
#pragma unroll
        for (int kg = 0; kg < KC / 4; kg++) {
            float4 x = make_float4(v[4 * kg], v[4 * kg + 1], v[4 * kg + 2], v[4 * kg + 3]);
            float4 h = make_float4(tf32_hi(x.x), tf32_hi(x.y), tf32_hi(x.z), tf32_hi(x.w));
            float4 l = make_float4(x.x - h.x, x.y - h.y, x.z - h.z, x.w - h.w);
            uint32_t off = kmaj_off(n, kg * 4, KC);
            *reinterpret_cast<float4 *>(hi + off) = h;
            *reinterpret_cast<float4 *>(lo + off) = l;
        }
    }
};

__global__ void __launch_bounds__(128) k_tc_dst_cols(DevGrid d, float *__restrict__ Y, const float *__restrict__ S1all,
                                                    const int64_t *__restrict__ s1off, const int *__restrict__ nopr1,
                                                    const double *__restrict__ p2r1, const double *__restrict__ p2r2,
                                                    double radcut, int seg0, int *__restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char *sm = smraw + ((1024 - (smem_u32(smraw) & 1023)) & 1023);
    int seg = seg0 + blockIdx.x;
    int g = seg / d.na, a = seg % d.na;
    int w = d.blk_wave[g];
    int nn = nopr1[w * d.na + a];
    const float *S1 = S1all + s1off[w * d.na + a];
    const int n1 = d.n1, n2 = d.n2;
    int col0 = blockIdx.y * COLS_BN;
    float *base = Y + (size_t)seg * n1 * n2;
    uint64_t *bars;
    uint32_t taddr;
    setup_cta(sm, COLS_BYTES, 4, COLS_BN, &bars, &taddr);
    const uint32_t idesc = idesc_tf32(128, COLS_BN);
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    bool ok = true;
    int nk = (nn + KC - 1) / KC;
    uint32_t sa = smem_u32(sm);
    // ---- GEMM 1: U = S1 * Y[:, cols] ----
    {
        uint32_t phase[2] = {0u, 0u};
        RowStage<128> sa;
        ColStage sb;
        sa.load(S1, nn, nn, nn, 0, 0);
        sb.load(base, n2, nn, 0, col0);
        for (int kc = 0; kc < nk; kc++) {
            int s = kc & 1;
            if (kc >= 2) {
                if (!mbar_wait(&bars[s], phase[s])) ok = false;
                phase[s] ^= 1u;
            }
            unsigned char *as = sm + COLS_A_OFF + s * 2 * A_PLANE;
            unsigned char *bs = sm + COLS_B_OFF + s * COLS_B1_STAGE;
            sa.store(as, as + A_PLANE);
            sb.store(bs, bs + COLS_B1_STAGE / 2);
            if (kc + 1 < nk) {
                sa.load(S1, nn, nn, nn, 0, (kc + 1) * KC);
                sb.load(base, n2, nn, (kc + 1) * KC, col0);
            }
            fence_async_smem();
            __syncthreads();
            if (threadIdx.x == 0 && ok) {
                fence_after_sync();
                uint32_t ah = smem_u32(as), al = ah + A_PLANE;
                uint32_t bh = smem_u32(bs), bl = bh + COLS_B1_STAGE / 2;
#pragma unroll
                for (int ks = 0; ks < KC / 8; ks++) {
                    uint32_t o = ks * 256;
                    uint64_t dah = sdesc(ah + o, 128, SBO), dal = sdesc(al + o, 128, SBO);
                    uint64_t dbh = sdesc(bh + o, 128, SBO), dbl = sdesc(bl + o, 128, SBO);
                    mma_tf32(taddr, dah, dbh, idesc, (kc > 0 || ks > 0) ? 1 : 0);
                    mma_tf32(taddr, dah, dbl, idesc, 1);
                    mma_tf32(taddr, dal, dbh, idesc, 1);
                }
                mma_commit(&bars[s]);
            }
        }
        int last = (nk - 1) & 1;
        if (!mbar_wait(&bars[last], phase[last])) ok = false;
        fence_after_sync();
    }
    // ---- scaling in k space; U (transposed, K-major in k) becomes the B operand ----
    {
        float *ut = reinterpret_cast<float *>(sm + COLS_A_OFF);     // 64 KB, A stages idle
        tmem_to_smem<COLS_BN>(taddr, ut);
        fence_before_sync();
        __syncthreads();
        fence_after_sync();
        const double *p1 = p2r1 + ((size_t)w * d.na + a) * n1;
        const double *p2 = p2r2 + ((size_t)w * d.na + a) * n2;
        const float divi = (float)(1.0 / (4.0 * (double)(nn + 1) * (double)(n2 + 1)));
        const float rc = (float)radcut;
        unsigned char *bh = sm + COLS_B_OFF, *bl = bh + COLS_B2 / 2;
        int n = threadIdx.x, col = col0 + n;
        float e2 = (col < n2) ? (float)p2[col] : 0.f;
        for (int mg = 0; mg < 128 / 4; mg++) {
            float u[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                int m = 4 * mg + i;
                float x = 0.f;
                if (m < nn && col < n2) {
                    float ek = (float)p1[m] + e2;
                    if (ek > rc) ek = rc;
                    x = tile_get(ut, COLS_BN, m, n) * ek * divi;
                }
                u[i] = x;
            }
            float4 h = make_float4(tf32_hi(u[0]), tf32_hi(u[1]), tf32_hi(u[2]), tf32_hi(u[3]));
            float4 l = make_float4(u[0] - h.x, u[1] - h.y, u[2] - h.z, u[3] - h.w);
            uint32_t off = kmaj_off(n, 4 * mg, 128);
            *reinterpret_cast<float4 *>(bh + off) = h;
            *reinterpret_cast<float4 *>(bl + off) = l;
        }
        fence_async_smem();
        __syncthreads();
    }
    // ---- GEMM 2: V = S1 * U ----
    {
        uint32_t phase[2] = {0u, 0u};
        const uint32_t sbo2 = (128 / 4) * 128;
        uint32_t bh = sa + COLS_B_OFF, bl = bh + COLS_B2 / 2;
        RowStage<128> st;
        st.load(S1, nn, nn, nn, 0, 0);
        for (int kc = 0; kc < nk; kc++) {
            int s = kc & 1;
            if (kc >= 2) {
                if (!mbar_wait(&bars[2 + s], phase[s])) ok = false;
                phase[s] ^= 1u;
            }
            unsigned char *as = sm + COLS_A_OFF + s * 2 * A_PLANE;
            st.store(as, as + A_PLANE);
            if (kc + 1 < nk) st.load(S1, nn, nn, nn, 0, (kc + 1) * KC);
            fence_async_smem();
            __syncthreads();
            if (threadIdx.x == 0 && ok) {
                fence_after_sync();
                uint32_t ah = smem_u32(as), al = ah + A_PLANE;
#pragma unroll
                for (int ks = 0; ks < KC / 8; ks++) {
                    uint32_t oa = ks * 256, ob = (kc * (KC / 8) + ks) * 256;
                    uint64_t dah = sdesc(ah + oa, 128, SBO), dal = sdesc(al + oa, 128, SBO);
                    uint64_t dbh = sdesc(bh + ob, 128, sbo2), dbl = sdesc(bl + ob, 128, sbo2);
                    mma_tf32(taddr, dah, dbh, idesc, (kc > 0 || ks > 0) ? 1 : 0);
                    mma_tf32(taddr, dah, dbl, idesc, 1);
                    mma_tf32(taddr, dal, dbh, idesc, 1);
                }
                mma_commit(&bars[2 + s]);
            }
        }
        int last = (nk - 1) & 1;
        if (!mbar_wait(&bars[2 + last], phase[last])) ok = false;
        fence_after_sync();
    }
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    {
        float *vt = reinterpret_cast<float *>(sm + COLS_B_OFF);
        tmem_to_smem<COLS_BN>(taddr, vt);
        __syncthreads();
        for (int m = warp; m < nn; m += 4) {
            float *row = base + (size_t)m * n2;
            for (int n = lane; n < COLS_BN; n += 32)
                if (col0 + n < n2) row[col0 + n] = tile_get(vt, COLS_BN, m, n);
        }
    }
    teardown_cta(taddr, COLS_BN);
}

}  // namespace tc

bool tc_dst_supported(Ctx &c)
{
    if (c.fp64 || !c.use_tc || c.k_dst == 3) return false;
    for (auto &t : c.waves)
        for (int a = 0; a < c.na; a++)
            if (t.nopr1[a] > 128) return false;
    return true;
}

void launch_tc_dst(Ctx &c, const float *X, float *Y, double *H, int g_begin, int g_end, int stage_base)
{
    using namespace tc;
    static bool attr = false;
    size_t smr = TileSmem<128>::BYTES + 2048, smc = COLS_BYTES + 2048;
    if (!attr) {
        cudaFuncSetAttribute(k_tc_dst_rows<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr);
        cudaFuncSetAttribute(k_tc_dst_rows<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr);
        cudaFuncSetAttribute(k_tc_dst_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc);
        attr = true;
    }
    int *err = c.d_tc_err;
    DevGrid d = devgrid(c);
    int ng = g_end - g_begin;
    int64_t row0 = (int64_t)g_begin * c.na * c.n1, nrows = (int64_t)ng * c.na * c.n1;
    dim3 gr((unsigned)((nrows + 127) / 128), (c.n2 + 127) / 128);
    stage_mark(c, stage_base + 0);
    k_tc_dst_rows<false><<<gr, 128, smr, c.stream>>>(d, X, (const float *)c.d_S2, Y, nullptr, c.d_nopr1, row0, nrows,
                                                     err);
    c.launches++;
    stage_mark(c, stage_base + 1);
    dim3 gc(ng * c.na, (c.n2 + COLS_BN - 1) / COLS_BN);
    k_tc_dst_cols<<<gc, 128, smc, c.stream>>>(d, Y, (const float *)c.d_S1, c.d_S1off, c.d_nopr1, c.d_p2r1, c.d_p2r2,
                                              c.grid.radcutmax, g_begin * c.na, err);
    c.launches++;
    stage_mark(c, stage_base + 2);
    k_tc_dst_rows<true><<<gr, 128, smr, c.stream>>>(d, Y, (const float *)c.d_S2, nullptr, H, c.d_nopr1, row0, nrows,
                                                    err);
    c.launches++;
}

}  // namespace mw3

// Self-test hook for the test suite: C = A Bt^T on device buffers with the
// tensor-core tile (BN = 128 or 256); returns 0, or 1 when an mbarrier wait ran
// out, or a CUDA error code + 100.
extern "C" int mw3_tc_gemm_selftest(const float *A, const float *Bt, float *C, int M, int N, int K, int bn)
{
    using namespace mw3::tc;
    int *err = nullptr;
    if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return 100;
    cudaMemset(err, 0, sizeof(int));
    dim3 grid((N + bn - 1) / bn, (M + 127) / 128);
    cudaError_t e;
    if (bn == 256) {
        size_t sm = TileSmem<256>::BYTES + 1024;
        cudaFuncSetAttribute(k_tc_gemm_test<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_tc_gemm_test<256><<<grid, 128, sm>>>(A, Bt, C, M, N, K, err);
    } else {
        size_t sm = TileSmem<128>::BYTES + 1024;
        cudaFuncSetAttribute(k_tc_gemm_test<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_tc_gemm_test<128><<<grid, 128, sm>>>(A, Bt, C, M, N, K, err);
    }
    e = cudaDeviceSynchronize();
    int h = 0;
    cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(err);
    if (e != cudaSuccess) return 100 + (int)e;
    return h;
}
