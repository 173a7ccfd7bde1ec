// Radial kinetic term of the mixed path (difs T-part, SRC/mod_Hphi_01y2.f:752-832)
// as ONE kernel per (block, angle) slab, everything between reading psi and
// writing H kept on chip (tensor memory holds the intermediate products, R up
// to 256 points as two 128-lane tiles).
//
// With Xs = psi on the slab [r1 < nopr1][R], the reference computes (RODFT00
// along R, along r1, k-space scaling, back along r1 and R)
//   H = S1 ((S1 Xs S2) o F) S2 ,   F[r1][R] = min(p2r1 + p2r2, radcut) / (4 (nopr1+1)(npun2+1)).
// Four 128 x 128 tensor-core GEMMs, oriented so that each result can be read
// out of tensor memory row by row (a thread owns one lane) and written back as
// the next GEMM's K-major operand without a transpose:
//   D1[R][r1] = S2 Xs^T            A = S2 (bulk copy)      B = Xs rows (global)
//   D2[R][r1] = D1 S1^T            A = D1 (tensor memory)  B = S1 (bulk copy)
//   D3[r1][R] = S1 (D2 o F^T)^T    A = S1 (bulk copy)      B = D2 o F^T (tensor memory)
//   D4[r1][R] = D3 S2              A = D3 (tensor memory)  B = S2 (bulk copy)
// so H[r1][R] = D4, written with lanes along r1 (stored points are r1-major runs).
// K streams in chunks of 32 through two shared-memory stages; the DST matrices
// are split on the host into TF32 hi/lo planes in the canonical K-major chunk
// layout and arrive by one bulk (TMA) copy per chunk.  3xTF32 products with
// FP32 accumulation as the other tensor-core kernels of the mixed path.
#include "mw3_internal.h"
#include "mw3_tc.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>

namespace mw3 {
namespace tc {

// R (npun2) up to 256: one or two 128-row tiles.  Each stage has a "big" slot
// for the operand that spans R (hi and lo planes of RB rows x 32 k, RB = 128
// or 256) and a "small" slot for the 128-row operand.
constexpr int D2_KC = 32;
constexpr uint32_t D2_SBO = (D2_KC / 4) * 128;    // 1 KB between 8-row groups
constexpr uint32_t D2_SMALL = 2 * 128 * 128;      // 32 KB: hi + lo, 128 rows x 32 k
constexpr uint32_t D2_BIGMAX = 2 * 256 * 128;     // 64 KB: hi + lo, 256 rows x 32 k
constexpr uint32_t D2_STAGE = D2_BIGMAX + D2_SMALL;
constexpr uint32_t D2_BYTES = 2 * D2_STAGE;       // 192 KB

struct Dst2Args {
    const float *X;               // rectangle [G][na][n1][n2]
    float *H;                     // H psi without V, FP32
    const float *planes;          // S2 (RB x RB) at 0, S1 of each length at s1off
    const int64_t *s1off;         // [W][na]
    const int *nopr1;             // [W][na]
    const float *p2r1f, *p2r2f;   // [W][na][n1], [W][na][n2]
    float radcut;
    const int *mapT;              // [na][n2][n1]
    const int64_t *foff;
    const int *blk_wave;
    int na, n1, n2, seg0;
    int *err;
};

// four values of one row into the hi plane at off and the lo plane lo_off further
__device__ __forceinline__ void d2_split4(unsigned char *hi, uint32_t lo_off, uint32_t off, float a, float b,
                                          float c, float d)
{
    float4 h = make_float4(tf32_hi(a), tf32_hi(b), tf32_hi(c), tf32_hi(d));
    float4 l = make_float4(a - h.x, b - h.y, c - h.z, d - h.w);
    *reinterpret_cast<float4 *>(hi + off) = h;
    *reinterpret_cast<float4 *>(hi + lo_off + off) = l;
}

// rows r < nn of the slab, K columns [32c, 32c+32): four float4 per thread;
// a quarter warp covers 8 rows of one 16-byte column group (one core matrix)
struct XStage {
    float4 v[4];
    __device__ __forceinline__ static void idx(int e, int &r, int &kg)
    {
        int rest = e >> 3;
        kg = rest & 7;
        r = (rest >> 3) * 8 + (e & 7);
    }
    __device__ __forceinline__ void load(const float *Xs, int n2, int nn, int c)
    {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            int r, kg;
            idx(threadIdx.x + 256 * i, r, kg);
            int k = c * D2_KC + kg * 4;
            float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
            if (r < nn) {
                const float *q = Xs + (size_t)r * n2 + k;
                if (k + 3 < n2 && (n2 & 3) == 0) {
                    x = __ldg(reinterpret_cast<const float4 *>(q));
                } else {
                    if (k < n2) x.x = __ldg(q);
                    if (k + 1 < n2) x.y = __ldg(q + 1);
                    if (k + 2 < n2) x.z = __ldg(q + 2);
                    if (k + 3 < n2) x.w = __ldg(q + 3);
                }
            }
            v[i] = x;
        }
    }
    __device__ __forceinline__ void store(unsigned char *dst) const
    {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            int r, kg;
            idx(threadIdx.x + 256 * i, r, kg);
            d2_split4(dst, D2_SMALL / 2, kmaj_off(r, kg * 4, D2_KC), v[i].x, v[i].y, v[i].z, v[i].w);
        }
    }
};

// Tensor memory (512 columns): D1 and D3 at [0, 256), D2 and D4 at [256, 512);
// D1/D2 hold R tile t at +128 t.
__global__ void __launch_bounds__(256, 1) k_tc_dst2d(Dst2Args p)
{
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char *sm = smraw + ((1024 - (smem_u32(smraw) & 1023)) & 1023);
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + D2_BYTES);   // [s] MMA of stage s, [2+s] its bulk copy
    uint32_t *slot = reinterpret_cast<uint32_t *>(bars + 4);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) tmem_alloc(slot, 512);
    if (threadIdx.x == 0) {
        for (int i = 0; i < 4; i++) mbar_init(&bars[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tb = *slot;
    const int na = p.na, n1 = p.n1, n2 = p.n2;
    const int NT = (n2 + 127) / 128;                    // R tiles
    const int RB = 128 * NT;
    const uint32_t big_lo = (uint32_t)RB * 128;         // lo plane offset in the big slot
    const int seg = p.seg0 + blockIdx.x;
    const int g = seg / na, a = seg % na, w = p.blk_wave[g];
    const int nn = p.nopr1[w * na + a];
    const float *S2p = p.planes;
    const float *S1p = p.planes + p.s1off[w * na + a];
    const float *Xs = p.X + (size_t)seg * n1 * n2;
    const int q4 = warp & 3, half = warp >> 2;
    const int m = q4 * 32 + lane;                       // the tensor-memory lane this thread reads
    const uint32_t lrow = tb + ((uint32_t)(q4 * 32) << 16);
    const float divi = 1.0f / (4.0f * (float)(nn + 1) * (float)(n2 + 1));
    const float *p1f = p.p2r1f + ((size_t)w * na + a) * n1;
    const int rR = 128 * half + m;                      // the R row this thread fills in GEMM 2 and 3
    const float e2 = (half < NT && rR < n2) ? p.p2r2f[((size_t)w * na + a) * n2 + rR] : 0.f;
    uint32_t ph_m[2] = {0u, 0u}, ph_c[2] = {0u, 0u};
    bool pend[2] = {false, false};
    bool bad = false, copy_out[2] = {false, false};
    int q = 0;
    XStage xs;

    for (int gi = 0; gi < 4; gi++) {
        const bool s2 = (gi == 0 || gi == 3);
        const int nk = s2 ? (n2 + D2_KC - 1) / D2_KC : (nn + D2_KC - 1) / D2_KC;
        // bulk operand: S2 chunk (RB rows) into the big slot, or S1 chunk into the small slot
        const size_t bulk_floats = s2 ? (size_t)2 * RB * D2_KC : (size_t)D2_SMALL / 4;
        const float *Sp = s2 ? S2p : S1p;
        if (gi > 0) {                                   // the previous GEMM must be complete
            for (int s = 0; s < 2; s++)
                if (pend[s]) {
                    if (!mbar_wait(&bars[s], ph_m[s])) bad = true;
                    ph_m[s] ^= 1u;
                    pend[s] = false;
                }
            fence_after_sync();
        } else {
            xs.load(Xs, n2, nn, 0);
        }
        for (int c = 0; c < nk; c++, q++) {
            const int s = q & 1;
            unsigned char *big = sm + s * D2_STAGE, *small = big + D2_BIGMAX;
            if (pend[s]) {                              // stage s is free once its MMAs are done
                if (!mbar_wait(&bars[s], ph_m[s])) bad = true;
                ph_m[s] ^= 1u;
                pend[s] = false;
                fence_after_sync();
            }
            if (threadIdx.x == 0) {
                mbar_expect_tx(&bars[2 + s], (uint32_t)(bulk_floats * 4));
                bulk_g2s(s2 ? big : small, Sp + (size_t)c * bulk_floats, (uint32_t)(bulk_floats * 4), &bars[2 + s]);
                copy_out[s] = true;
            }
            if (gi == 0) {
                // B = Xs rows (r1) into the small slot
                xs.store(small);
                if (c + 1 < nk) xs.load(Xs, n2, nn, c + 1);
            } else if (gi == 1 || gi == 2) {
                // A = D1 (gi 1) or B = D2 o F^T (gi 2): RB rows (R) into the big slot; warp half = R tile
                if (half < NT) {
                    float v[32];
                    const uint32_t src = (gi == 1 ? 0u : 256u) + 128u * half + (uint32_t)(c * D2_KC);
                    tmem_ld32(lrow + src, v);
                    if (gi == 2) {
#pragma unroll
                        for (int i = 0; i < 32; i++) {
                            int k = c * D2_KC + i;
                            float ek = 0.f;
                            if (k < nn && rR < n2) {
                                ek = __ldg(p1f + k) + e2;
                                if (ek > p.radcut) ek = p.radcut;
                            }
                            v[i] = v[i] * ek * divi;
                        }
                    }
#pragma unroll
                    for (int j = 0; j < 8; j++)
                        d2_split4(big, big_lo, kmaj_off(rR, 4 * j, D2_KC), v[4 * j], v[4 * j + 1], v[4 * j + 2],
                                  v[4 * j + 3]);
                }
            } else {
                // A = D3 rows (r1) into the small slot, the two warp halves 16 columns each
                float v[16];
                const int k0 = c * D2_KC + 16 * half;
                tmem_ld16(lrow + (uint32_t)k0, v);
#pragma unroll
                for (int j = 0; j < 4; j++)
                    d2_split4(small, D2_SMALL / 2, kmaj_off(m, 16 * half + 4 * j, D2_KC), v[4 * j], v[4 * j + 1],
                              v[4 * j + 2], v[4 * j + 3]);
            }
            fence_async_smem();
            fence_before_sync();
            if (__syncthreads_or(bad)) goto done;
            if (threadIdx.x == 0) {
                if (!mbar_wait(&bars[2 + s], ph_c[s])) bad = true;
                copy_out[s] = false;
                fence_after_sync();
                if (!bad) {
                    const uint32_t bg = smem_u32(big), sl = smem_u32(small);
#pragma unroll
                    for (int ks = 0; ks < D2_KC / 8; ks++) {
                        const uint32_t o = ks * 256;
                        const int acc0 = (c > 0 || ks > 0) ? 1 : 0;
                        if (gi <= 1) {
                            // M = 128 per R tile, N = 128 (r1): A = big (R rows), B = small
                            const uint32_t idesc = idesc_tf32(128, 128);
                            uint64_t dbh = sdesc(sl + o, 128, D2_SBO), dbl = sdesc(sl + D2_SMALL / 2 + o, 128, D2_SBO);
                            for (int t = 0; t < NT; t++) {
                                uint32_t at = bg + (uint32_t)t * 16 * D2_SBO;
                                uint64_t dah = sdesc(at + o, 128, D2_SBO), dal = sdesc(at + big_lo + o, 128, D2_SBO);
                                uint32_t d = tb + (gi == 0 ? 0u : 256u) + 128u * t;
                                mma_tf32(d, dah, dbh, idesc, acc0);
                                mma_tf32(d, dah, dbl, idesc, 1);
                                mma_tf32(d, dal, dbh, idesc, 1);
                            }
                        } else {
                            // M = 128 (r1), N = RB (R): A = small, B = big
                            const uint32_t idesc = idesc_tf32(128, RB);
                            uint64_t dah = sdesc(sl + o, 128, D2_SBO), dal = sdesc(sl + D2_SMALL / 2 + o, 128, D2_SBO);
                            uint64_t dbh = sdesc(bg + o, 128, D2_SBO), dbl = sdesc(bg + big_lo + o, 128, D2_SBO);
                            uint32_t d = tb + (gi == 2 ? 0u : 256u);
                            mma_tf32(d, dah, dbh, idesc, acc0);
                            mma_tf32(d, dah, dbl, idesc, 1);
                            mma_tf32(d, dal, dbh, idesc, 1);
                        }
                    }
                }
                mma_commit(&bars[s]);
            }
            ph_c[s] ^= 1u;
            pend[s] = true;
        }
    }
    for (int s = 0; s < 2; s++)
        if (pend[s]) {
            if (!mbar_wait(&bars[s], ph_m[s])) bad = true;
            ph_m[s] ^= 1u;
            pend[s] = false;
        }
    fence_after_sync();
    if (__syncthreads_or(bad)) goto done;
    // ---- H at the stored points: D4 lane = r1, column = R ----
    {
        const int *mT = p.mapT + (size_t)a * n2 * n1;
        const int64_t fo = p.foff[seg];
        for (int cc = 0; cc < RB / 32; cc++) {
            const int c0 = (RB / 2) * half + 16 * cc;
            float v[16];
            tmem_ld16(lrow + 256u + (uint32_t)c0, v);
            int idx[16];
#pragma unroll
            for (int i = 0; i < 16; i++) {
                int r2 = c0 + i;
                idx[i] = (m < nn && r2 < n2) ? __ldg(mT + (size_t)r2 * n1 + m) : -1;
            }
#pragma unroll
            for (int i = 0; i < 16; i++)
                if (idx[i] >= 0) p.H[fo + idx[i]] = v[i];
        }
    }
done:
    if (bad && threadIdx.x == 0) atomicExch(p.err, 1);
    if (threadIdx.x == 0) {
        // a bulk copy issued before a failed wait must land before the CTA exits
        for (int s = 0; s < 2; s++)
            if (copy_out[s]) mbar_wait(&bars[2 + s], ph_c[s]);
    }
    for (int s = 0; s < 2; s++)
        if (pend[s]) mbar_wait(&bars[s], ph_m[s]);
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tb, 512);
}

}  // namespace tc

namespace {

float tf32_round_nearest(float x)
{
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;      // nearest, ties away from zero (cvt.rna)
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

// one n x n DST-I matrix as K-chunks of 32: each chunk [hi plane][lo plane] of
// rows x 32 k in the canonical K-major layout, zero padded to rows x rows
void append_planes(std::vector<float> &out, const std::vector<double> &S, int n, int rows)
{
    size_t base = out.size();
    const size_t plane = (size_t)rows * tc::D2_KC;
    out.resize(base + (size_t)(rows / tc::D2_KC) * 2 * plane, 0.f);
    for (int r = 0; r < n; r++)
        for (int k = 0; k < n; k++) {
            float x = (float)S[(size_t)r * n + k], h = tf32_round_nearest(x), l = x - h;
            int c = k / tc::D2_KC, kk = k % tc::D2_KC;
            size_t o = (size_t)((r & 7) * 16 + (r >> 3) * tc::D2_SBO + (kk & 3) * 4 + (kk >> 2) * 128) / 4;
            out[base + (size_t)c * 2 * plane + o] = h;
            out[base + (size_t)c * 2 * plane + plane + o] = l;
        }
}

template <typename V>
int upload_vec(Ctx &c, V **dst, const std::vector<V> &v)
{
    *dst = nullptr;
    size_t bytes = sizeof(V) * std::max<size_t>(v.size(), 1);
    cudaError_t e = cudaMalloc((void **)dst, bytes);
    if (e == cudaSuccess) {
        c.allocs.push_back(*dst);
        if (!v.empty()) e = cudaMemcpy(*dst, v.data(), sizeof(V) * v.size(), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        c.err = std::string("fused DST tables: ") + cudaGetErrorString(e);
        return MW3_ERR_CUDA;
    }
    return MW3_OK;
}

}  // namespace

std::vector<double> dst_matrix(int n);

// Tables of the fused radial kernel; c.use_tc_dst2d stays false when the shape
// is outside it (npun2 > 256 or an r1 DST length above 128: the three-kernel
// tensor-core path or the CUDA-core path runs instead).
int build_tc_dst2d(Ctx &c)
{
    c.use_tc_dst2d = false;
    if (c.fp64 || !c.use_tc || c.n2 > 256) return MW3_OK;
    const int na = c.na, W = (int)c.waves.size();
    for (auto &t : c.waves)
        for (int a = 0; a < na; a++)
            if (t.nopr1[a] > 128 || t.nopr1[a] < 1) return MW3_OK;
    std::vector<float> planes;
    append_planes(planes, dst_matrix(c.n2), c.n2, 128 * ((c.n2 + 127) / 128));
    std::map<int, int64_t> off;
    std::vector<int64_t> s1off((size_t)W * na);
    std::vector<float> p1f((size_t)W * na * c.n1), p2f((size_t)W * na * c.n2);
    for (int w = 0; w < W; w++) {
        const WaveTables &t = c.waves[w];
        for (int a = 0; a < na; a++) {
            int nn = t.nopr1[a];
            auto it = off.find(nn);
            if (it == off.end()) {
                int64_t o = (int64_t)planes.size();
                append_planes(planes, dst_matrix(nn), nn, 128);
                it = off.emplace(nn, o).first;
            }
            s1off[(size_t)w * na + a] = it->second;
        }
        for (size_t i = 0; i < t.p2r1.size(); i++) p1f[(size_t)w * na * c.n1 + i] = (float)t.p2r1[i];
        for (size_t i = 0; i < t.p2r2.size(); i++) p2f[(size_t)w * na * c.n2 + i] = (float)t.p2r2[i];
    }
    int rc;
    if ((rc = upload_vec(c, &c.d_dst_planes, planes))) return rc;
    if ((rc = upload_vec(c, &c.d_dst_s1off, s1off))) return rc;
    if ((rc = upload_vec(c, &c.d_p2r1f, p1f))) return rc;
    if ((rc = upload_vec(c, &c.d_p2r2f, p2f))) return rc;
    c.use_tc_dst2d = true;
    return MW3_OK;
}

void launch_tc_dst2d(Ctx &c, const float *X, float *H, int g_begin, int g_end)
{
    using namespace tc;
    static bool attr = false;
    const size_t smem = D2_BYTES + 64 + 1024;
    if (!attr) {
        cudaFuncSetAttribute(k_tc_dst2d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    int nseg = (g_end - g_begin) * c.na;
    if (nseg <= 0) return;
    Dst2Args p;
    p.X = X; p.H = H;
    p.planes = c.d_dst_planes; p.s1off = c.d_dst_s1off; p.nopr1 = c.d_nopr1;
    p.p2r1f = c.d_p2r1f; p.p2r2f = c.d_p2r2f; p.radcut = (float)c.grid.radcutmax;
    p.mapT = c.d_mapT; p.foff = c.d_foff; p.blk_wave = c.d_blk_wave;
    p.na = c.na; p.n1 = c.n1; p.n2 = c.n2; p.seg0 = g_begin * c.na;
    p.err = c.d_tc_err;
    k_tc_dst2d<<<nseg, 256, smem, c.stream>>>(p);
    c.launches++;
}

}  // namespace mw3
