// Neural radiance cache kernels (no counterpart in the reference; see nrc.h).
//
// Network evaluation is a fully fused MLP on the tensor cores: each warp takes 16 rows,
// every layer is mma.sync m16n8k16 (BF16 x BF16 -> FP32) against weights held in shared
// memory as pre-packed B fragments, and a layer's FP32 accumulators become the next
// layer's A fragments in registers (the m16n8 accumulator of two adjacent n-tiles has the
// layout of one m16k16 A fragment), so activations never leave the register file during
// inference. Training runs forward + relative-L2 loss + backward in the same fused kernel
// (activations kept in shared memory for the ReLU masks), writes layer inputs X_l and
// pre-activation gradients dY_l for the weight-gradient GEMMs dW_l = X_l^T dY_l (a second
// tensor-core kernel, split over the batch), scatters the encoding gradient into the hash
// table with float2 atomics, and finishes with FP32 Adam over all parameters.
#include "nrc.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <vector>

namespace bt {

namespace {

constexpr int NRC_BLOCK = 128;           // 4 warps
constexpr int NRC_WARPS = NRC_BLOCK / 32;
constexpr int X0_STRIDE = 88;            // bf16 elements per input row in shared memory
constexpr int XH_STRIDE = 72;            // bf16 elements per hidden row in shared memory

// weight matrix shapes and offsets (row-major K x N in the FP32 master copy)
__host__ __device__ constexpr int layer_k(int l) { return l == 0 ? NRC_IN : NRC_WIDTH; }
__host__ __device__ constexpr int layer_n(int l) { return l == NRC_LAYERS - 1 ? NRC_OUT : NRC_WIDTH; }
__host__ __device__ constexpr int w_offset(int l)
{
    int o = 0;
    for(int j = 0; j < l; ++j)
        o += layer_k(j) * layer_n(j);
    return o;
}
// packed fragments: forward B = W (K x N); backward B = W^T (N x K), for layer 0 only the
// 32 hash-feature columns of dX are needed
__host__ __device__ constexpr int bwd_n(int l) { return l == 0 ? 32 : layer_k(l); }
__host__ __device__ constexpr int fwd_base(int l)
{
    int o = 0;
    for(int j = 0; j < l; ++j)
        o += (layer_k(j) / 16) * (layer_n(j) / 8) * 32;
    return o;
}
__host__ __device__ constexpr int bwd_base(int l)
{
    int o = 0;
    for(int j = 0; j < l; ++j)
        o += (layer_n(j) / 16) * (bwd_n(j) / 8) * 32;
    return o;
}
constexpr int FWD_PACKED = fwd_base(NRC_LAYERS);  // uint2 entries
constexpr int BWD_PACKED = bwd_base(NRC_LAYERS);
// act / dact layer offsets in elements per row
__host__ __device__ constexpr int act_cols_before(int l)
{
    int o = 0;
    for(int j = 0; j < l; ++j)
        o += layer_k(j);
    return o;
}
__host__ __device__ constexpr int dact_cols_before(int l)
{
    int o = 0;
    for(int j = 0; j < l; ++j)
        o += layer_n(j);
    return o;
}
constexpr int ACT_COLS = act_cols_before(NRC_LAYERS);
constexpr int DACT_COLS = dact_cols_before(NRC_LAYERS);

struct LevelInfo
{
    float res;
    uint32_t stride;   // dense grid stride, 0 for hashed levels
};
__constant__ LevelInfo c_levels[NRC_LEVELS];

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ float2 unpack_bf16(uint32_t v)
{
    const __nv_bfloat162 b = *reinterpret_cast<const __nv_bfloat162 *>(&v);
    return __bfloat1622float2(b);
}

__device__ __forceinline__ void mma(float (&d)[4], const uint32_t (&a)[4], uint2 b)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// ------------------------------------------------------------------ encoding

// real spherical harmonics of bands 0..3 (16 values) of a unit vector
__device__ __forceinline__ void sh16(V3 d, float *o)
{
    const float x = d.x, y = d.y, z = d.z, xx = x * x, yy = y * y, zz = z * z;
    o[0] = 0.28209479177387814f;
    o[1] = -0.48860251190291987f * y;
    o[2] = 0.48860251190291987f * z;
    o[3] = -0.48860251190291987f * x;
    o[4] = 1.0925484305920792f * x * y;
    o[5] = -1.0925484305920792f * y * z;
    o[6] = 0.94617469575755997f * zz - 0.31539156525251999f;
    o[7] = -1.0925484305920792f * x * z;
    o[8] = 0.54627421529603959f * (xx - yy);
    o[9] = 0.59004358992664352f * y * (-3.0f * xx + yy);
    o[10] = 2.8906114426405538f * x * y * z;
    o[11] = 0.45704579946446572f * y * (1.0f - 5.0f * zz);
    o[12] = 0.3731763325901154f * z * (5.0f * zz - 3.0f);
    o[13] = 0.45704579946446572f * x * (1.0f - 5.0f * zz);
    o[14] = 1.4453057213202769f * z * (xx - yy);
    o[15] = 0.59004358992664352f * x * (-xx + 3.0f * yy);
}

__device__ __forceinline__ V3 nrc_unit_pos(const NrcDev &D, const float *q)
{
    V3 p((q[0] - D.bbox_min[0]) * D.bbox_inv_extent[0], (q[1] - D.bbox_min[1]) * D.bbox_inv_extent[1],
         (q[2] - D.bbox_min[2]) * D.bbox_inv_extent[2]);
    p.x = fminf(fmaxf(p.x, 0.0f), 1.0f);
    p.y = fminf(fmaxf(p.y, 0.0f), 1.0f);
    p.z = fminf(fmaxf(p.z, 0.0f), 1.0f);
    return p;
}

// corners of one level: table indices and trilinear weights
__device__ __forceinline__ void level_corners(V3 p, int l, uint32_t *idx, float *w)
{
    const LevelInfo L = c_levels[l];
    const float x = p.x * L.res, y = p.y * L.res, z = p.z * L.res;
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    const float tx = x - fx, ty = y - fy, tz = z - fz;
    const uint32_t ix = static_cast<uint32_t>(fx), iy = static_cast<uint32_t>(fy), iz = static_cast<uint32_t>(fz);
#pragma unroll
    for(int c = 0; c < 8; ++c)
    {
        const uint32_t cx = ix + (c & 1), cy = iy + ((c >> 1) & 1), cz = iz + ((c >> 2) & 1);
        uint32_t h;
        if(L.stride)
            h = cx + cy * L.stride + cz * L.stride * L.stride;
        else
            h = (cx * 1u) ^ (cy * 2654435761u) ^ (cz * 805459861u);  // Instant-NGP spatial hash
        idx[c] = (h & (NRC_TABLE - 1)) + static_cast<uint32_t>(l) * NRC_TABLE;
        w[c] = ((c & 1) ? tx : 1.0f - tx) * (((c >> 1) & 1) ? ty : 1.0f - ty) * (((c >> 2) & 1) ? tz : 1.0f - tz);
    }
}

// one half of a row's 80 inputs: half 0 = hash levels 0..7 and SH(direction); half 1 =
// hash levels 8..15, SH(normal), roughness, albedo, the constant 1 and zero padding
__device__ __forceinline__ void encode_half(const NrcDev &D, const float *q, int half, __nv_bfloat16 *row)
{
    const V3 p = nrc_unit_pos(D, q);
    for(int l = half * 8; l < half * 8 + 8; ++l)
    {
        uint32_t idx[8];
        float w[8];
        level_corners(p, l, idx, w);
        float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
        for(int c = 0; c < 8; ++c)
        {
            const float2 f = __half22float2(D.hash[idx[c]]);
            f0 += w[c] * f.x;
            f1 += w[c] * f.y;
        }
        row[l * 2] = __float2bfloat16_rn(f0);
        row[l * 2 + 1] = __float2bfloat16_rn(f1);
    }
    float sh[16];
    if(half == 0)
    {
        sh16(normalize(V3(q[3], q[4], q[5])), sh);
        for(int k = 0; k < 16; ++k)
            row[32 + k] = __float2bfloat16_rn(sh[k]);
    }
    else
    {
        sh16(normalize(V3(q[6], q[7], q[8])), sh);
        for(int k = 0; k < 16; ++k)
            row[48 + k] = __float2bfloat16_rn(sh[k]);
        row[64] = __float2bfloat16_rn(q[9]);
        row[65] = __float2bfloat16_rn(q[10]);
        row[66] = __float2bfloat16_rn(q[11]);
        row[67] = __float2bfloat16_rn(q[12]);
        row[68] = __float2bfloat16_rn(1.0f);
        for(int k = 69; k < NRC_IN; ++k)
            row[k] = __float2bfloat16_rn(0.0f);
    }
}

// ------------------------------------------------------------------ fused MLP pieces

// A fragments of a 16 x 16 tile from a bf16 row-major shared tile
__device__ __forceinline__ void load_a(const __nv_bfloat16 *tile, int stride, int kt, int lane, uint32_t (&a)[4])
{
    const int g = lane >> 2, t = lane & 3;
    const uint32_t *r0 = reinterpret_cast<const uint32_t *>(tile + g * stride + kt * 16 + 2 * t);
    const uint32_t *r1 = reinterpret_cast<const uint32_t *>(tile + (g + 8) * stride + kt * 16 + 2 * t);
    a[0] = r0[0];
    a[1] = r1[0];
    a[2] = r0[4];
    a[3] = r1[4];
}

// accumulators of n-tiles (2k, 2k+1) -> A fragment of k-tile k, with ReLU
__device__ __forceinline__ void acc_to_a_relu(const float (&c0)[4], const float (&c1)[4], uint32_t (&a)[4])
{
    a[0] = pack_bf16(fmaxf(c0[0], 0.0f), fmaxf(c0[1], 0.0f));
    a[1] = pack_bf16(fmaxf(c0[2], 0.0f), fmaxf(c0[3], 0.0f));
    a[2] = pack_bf16(fmaxf(c1[0], 0.0f), fmaxf(c1[1], 0.0f));
    a[3] = pack_bf16(fmaxf(c1[2], 0.0f), fmaxf(c1[3], 0.0f));
}

// store A fragments of k-tile kt into a bf16 row-major tile
__device__ __forceinline__ void store_a(__nv_bfloat16 *tile, int stride, int kt, int lane, const uint32_t (&a)[4])
{
    const int g = lane >> 2, t = lane & 3;
    uint32_t *r0 = reinterpret_cast<uint32_t *>(tile + g * stride + kt * 16 + 2 * t);
    uint32_t *r1 = reinterpret_cast<uint32_t *>(tile + (g + 8) * stride + kt * 16 + 2 * t);
    r0[0] = a[0];
    r1[0] = a[1];
    r0[4] = a[2];
    r1[4] = a[3];
}

__device__ __forceinline__ void load_weights(const uint2 *src, uint2 *dst, int count)
{
    for(int i = threadIdx.x; i < count; i += blockDim.x)
        dst[i] = src[i];
}

// hidden layers 1..4 (64 -> 64) on A fragments a[4 k-tiles]; writes the next A fragments
__device__ __forceinline__ void hidden_layer(const uint2 *sw, int l, int lane, uint32_t (&a)[4][4])
{
    float acc[8][4];
#pragma unroll
    for(int nt = 0; nt < 8; ++nt)
        acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
    const uint2 *w = sw + fwd_base(l);
#pragma unroll
    for(int kt = 0; kt < 4; ++kt)
#pragma unroll
        for(int nt = 0; nt < 8; ++nt)
            mma(acc[nt], a[kt], w[(kt * 8 + nt) * 32 + lane]);
#pragma unroll
    for(int kt = 0; kt < 4; ++kt)
        acc_to_a_relu(acc[2 * kt], acc[2 * kt + 1], a[kt]);
}

// ------------------------------------------------------------------ inference

__global__ void __launch_bounds__(NRC_BLOCK) k_nrc_infer(NrcDev D, const float *__restrict__ queries, uint32_t n,
                                                         float *__restrict__ out)
{
    extern __shared__ uint4 smem_raw[];
    uint2 *sw = reinterpret_cast<uint2 *>(smem_raw);
    __nv_bfloat16 *sx = reinterpret_cast<__nv_bfloat16 *>(sw + FWD_PACKED);
    load_weights(D.w_fwd, sw, FWD_PACKED);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __nv_bfloat16 *x0 = sx + warp * 16 * X0_STRIDE;
    const uint32_t tiles = (n + 15) / 16;
    for(uint32_t tile = blockIdx.x * NRC_WARPS + warp; tile < tiles; tile += gridDim.x * NRC_WARPS)
    {
        const uint32_t row = tile * 16 + (lane & 15);
        float q[NRC_QUERY_FLOATS];
        if(row < n)
            for(int k = 0; k < NRC_QUERY_FLOATS; ++k)
                q[k] = queries[static_cast<size_t>(row) * NRC_QUERY_FLOATS + k];
        else
            for(int k = 0; k < NRC_QUERY_FLOATS; ++k)
                q[k] = k == 5 || k == 8 ? 1.0f : 0.0f;
        encode_half(D, q, lane >> 4, x0 + (lane & 15) * X0_STRIDE);
        __syncwarp();
        // layer 0: 80 -> 64
        uint32_t a[4][4];
        {
            float acc[8][4];
#pragma unroll
            for(int nt = 0; nt < 8; ++nt)
                acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
            for(int kt = 0; kt < 5; ++kt)
            {
                uint32_t ax[4];
                load_a(x0, X0_STRIDE, kt, lane, ax);
#pragma unroll
                for(int nt = 0; nt < 8; ++nt)
                    mma(acc[nt], ax, sw[(kt * 8 + nt) * 32 + lane]);
            }
#pragma unroll
            for(int kt = 0; kt < 4; ++kt)
                acc_to_a_relu(acc[2 * kt], acc[2 * kt + 1], a[kt]);
        }
        __syncwarp();
#pragma unroll 1
        for(int l = 1; l < NRC_LAYERS - 1; ++l)
            hidden_layer(sw, l, lane, a);
        // output layer: 64 -> 16 (3 used)
        float o[2][4] = { { 0, 0, 0, 0 }, { 0, 0, 0, 0 } };
        const uint2 *w5 = sw + fwd_base(NRC_LAYERS - 1);
#pragma unroll
        for(int kt = 0; kt < 4; ++kt)
        {
            mma(o[0], a[kt], w5[(kt * 2 + 0) * 32 + lane]);
            mma(o[1], a[kt], w5[(kt * 2 + 1) * 32 + lane]);
        }
        // n-tile 0 holds outputs 0..7: thread (g, t) has rows g, g + 8, columns 2t, 2t + 1
        const int g = lane >> 2, t = lane & 3;
        if(t < 2)
        {
            const uint32_t r0 = tile * 16 + g, r1 = r0 + 8;
            if(r0 < n)
            {
                out[static_cast<size_t>(r0) * 4 + 2 * t] = o[0][0];
                if(t == 0)
                    out[static_cast<size_t>(r0) * 4 + 1] = o[0][1];
            }
            if(r1 < n)
            {
                out[static_cast<size_t>(r1) * 4 + 2 * t] = o[0][2];
                if(t == 0)
                    out[static_cast<size_t>(r1) * 4 + 1] = o[0][3];
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ inference on tcgen05
//
// The same network on the 5th-generation tensor cores. A block of 1024 threads holds the
// weights (45 KB) in shared memory once and runs eight independent groups of 128
// threads; each group takes 128 queries at a time: every thread encodes one query
// (16 hash levels, the two SH bands, the material inputs) straight into shared memory in
// the UMMA canonical K-major layout (8-row x 16-byte core matrices), one thread issues
// each layer as tcgen05.mma (M = 128, N = 64 or 16, K = 16 per instruction, BF16 x BF16
// -> FP32) into the group's 64 tensor-memory columns, and the group's four warps read the
// accumulator back with tcgen05.ld (warp w: lanes 32 (w % 4)..), apply ReLU, round to
// BF16 and write the next layer's operand over the previous one. The groups run out of
// step, so one group's hash gathers overlap another's MMAs; 32 warps per SM keep the
// gathers in flight. Every wait on an MMA completion barrier is bounded; on a timeout the
// group records an error and leaves, and the block releases its tensor memory.

constexpr int TC_GROUPS = 8;
constexpr int TC_ROWS = 128;                              // rows per group tile (MMA M)
constexpr int TC_BLOCK = TC_ROWS * TC_GROUPS;             // 1024 threads, one block per SM
constexpr uint32_t TC_GROUP_COLS = 64;                    // FP32 accumulator columns per group
constexpr uint32_t TC_TMEM_COLS = TC_GROUP_COLS * TC_GROUPS;  // all 512 columns of the SM
constexpr uint32_t TC_W_BYTES = NRC_WEIGHTS * 2;          // all layers, canonical layout
constexpr uint32_t TC_A_BYTES = TC_ROWS * NRC_IN * 2;     // one group's operand (80 columns at most)

// byte offset of layer l in the canonical weight image: W_l^T as N x K, K-major
__host__ __device__ constexpr uint32_t tc_w_offset(int l) { return static_cast<uint32_t>(w_offset(l)) * 2u; }
// byte offset of element (row r, column k) of an R x K K-major operand in core matrices:
// 16 bytes of 8 consecutive k per row, 8 rows per 128-byte core matrix, core matrices
// along K adjacent (128 bytes apart), 8-row groups K * 16 bytes apart
__host__ __device__ constexpr uint32_t tc_offset(int r, int k, int K)
{
    return static_cast<uint32_t>((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor, no swizzle: start, leading (K-direction core matrix
// stride) and stride (8-row group stride) byte offsets, descriptor version 1
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return static_cast<uint64_t>((saddr >> 4) & 0x3fffu) | (static_cast<uint64_t>((lbo >> 4) & 0x3fffu) << 16) |
           (static_cast<uint64_t>((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
           (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                 :
                 : "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
                 : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// wait for phase `parity` of the barrier, at most ~1 s; false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity)
{
    const uint64_t t0 = global_ns();
    for(uint32_t it = 0;; ++it)
    {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done)
                     : "r"(mbar), "r"(parity)
                     : "memory");
        if(done)
            return true;
        if((it & 1023u) == 1023u && global_ns() - t0 > 1000000000ull)
            return false;
        if(it > 64)
            __nanosleep(32);
    }
}

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes (one row per thread)
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                 "[%16];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for(int k = 0; k < 16; ++k)
        v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void tc_ld4(uint32_t taddr, float (&v)[4])
{
    uint32_t r[4];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for(int k = 0; k < 4; ++k)
        v[k] = __uint_as_float(r[k]);
}

// a query's 80 inputs (the columns of encode_half) written as the ten 16-byte chunks of
// row m of a canonical 128 x 80 operand
__device__ __forceinline__ void encode_row_tc(const NrcDev &D, const float *q, unsigned char *a, int m)
{
    const V3 p = nrc_unit_pos(D, q);
    unsigned char *row = a + tc_offset(m, 0, NRC_IN);
#pragma unroll 1
    for(int chunk = 0; chunk < 4; ++chunk)
    {
        // levels 4 chunk .. 4 chunk + 3: columns 8 chunk .. 8 chunk + 7
        uint32_t w4[4];
#pragma unroll
        for(int j = 0; j < 4; ++j)
        {
            uint32_t idx[8];
            float w[8];
            level_corners(p, chunk * 4 + j, idx, w);
            float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
            for(int c = 0; c < 8; ++c)
            {
                const float2 f = __half22float2(D.hash[idx[c]]);
                f0 += w[c] * f.x;
                f1 += w[c] * f.y;
            }
            w4[j] = pack_bf16(f0, f1);
        }
        *reinterpret_cast<uint4 *>(row + chunk * 128) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
    }
#pragma unroll 1
    for(int half = 0; half < 2; ++half)
    {
        // columns 32..47: SH of the direction to the viewer; 48..63: SH of the normal
        float sh[16];
        sh16(normalize(half == 0 ? V3(q[3], q[4], q[5]) : V3(q[6], q[7], q[8])), sh);
        unsigned char *c = row + (4 + 2 * half) * 128;
        *reinterpret_cast<uint4 *>(c) = make_uint4(pack_bf16(sh[0], sh[1]), pack_bf16(sh[2], sh[3]),
                                                   pack_bf16(sh[4], sh[5]), pack_bf16(sh[6], sh[7]));
        *reinterpret_cast<uint4 *>(c + 128) = make_uint4(pack_bf16(sh[8], sh[9]), pack_bf16(sh[10], sh[11]),
                                                         pack_bf16(sh[12], sh[13]), pack_bf16(sh[14], sh[15]));
    }
    // columns 64..79: roughness, albedo, the constant 1, zero padding
    *reinterpret_cast<uint4 *>(row + 8 * 128) =
        make_uint4(pack_bf16(q[9], q[10]), pack_bf16(q[11], q[12]), pack_bf16(1.0f, 0.0f), 0u);
    *reinterpret_cast<uint4 *>(row + 9 * 128) = make_uint4(0u, 0u, 0u, 0u);
}

// barrier over the 128 threads of group g (named barrier 1 + g), returning whether every
// thread passed `pred`
__device__ __forceinline__ bool group_sync_and(int g, bool pred)
{
    uint32_t r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
                 "bar.red.and.pred q, %2, 128, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
                 : "=r"(r)
                 : "r"(pred ? 1u : 0u), "r"(1 + g)
                 : "memory");
    return r != 0;
}

__device__ __forceinline__ void group_sync(int g) { asm volatile("bar.sync %0, 128;\n" ::"r"(1 + g) : "memory"); }

__global__ void __launch_bounds__(TC_BLOCK, 1)
    k_nrc_infer_tc(NrcDev D, const float *__restrict__ queries, uint32_t n, float *__restrict__ out)
{
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char *sw = tc_smem;                                   // weights, canonical layout per layer
    uint64_t *mbar = reinterpret_cast<uint64_t *>(tc_smem + TC_W_BYTES + TC_GROUPS * TC_A_BYTES);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + TC_GROUPS);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = tid / TC_ROWS, m = tid % TC_ROWS;               // group, row of the group's tile
    unsigned char *sa = tc_smem + TC_W_BYTES + g * TC_A_BYTES;     // the group's operand

    // weights into shared memory (16-byte copies), barrier init, tensor-memory allocation
    for(uint32_t i = tid; i < TC_W_BYTES / 16; i += TC_BLOCK)
        reinterpret_cast<uint4 *>(sw)[i] = reinterpret_cast<const uint4 *>(D.w_tc)[i];
    if(tid < TC_GROUPS)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(mbar + tid)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if(warp == 0)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(tmem_slot)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot + static_cast<uint32_t>(g) * TC_GROUP_COLS;
    const uint32_t mb = smem_addr(mbar + g);
    const uint32_t a_addr = smem_addr(sa), w_addr = smem_addr(sw);
    // this warp's TMEM lane quarter; the row it reads back
    const uint32_t lane_base = static_cast<uint32_t>(32 * (warp & 3)) << 16;
    const int erow = 32 * (warp & 3) + lane;
    uint32_t phase = 0;
    bool ok = true;

    const uint32_t tiles = (n + TC_ROWS - 1) / TC_ROWS;
    for(uint32_t tile = blockIdx.x * TC_GROUPS + g; tile < tiles && ok; tile += gridDim.x * TC_GROUPS)
    {
        const uint32_t row = tile * TC_ROWS + m;
        float q[NRC_QUERY_FLOATS];
        if(row < n)
            for(int k = 0; k < NRC_QUERY_FLOATS; ++k)
                q[k] = queries[static_cast<size_t>(row) * NRC_QUERY_FLOATS + k];
        else
            for(int k = 0; k < NRC_QUERY_FLOATS; ++k)
                q[k] = k == 5 || k == 8 ? 1.0f : 0.0f;
        encode_row_tc(D, q, sa, m);
        fence_async_smem();
        group_sync(g);

        for(int l = 0; l < NRC_LAYERS && ok; ++l)
        {
            const int K = layer_k(l), N = layer_n(l);
            if(m == 0)
            {
                tc_fence_after();
                const uint32_t sbo = static_cast<uint32_t>(K * 16);
                for(int ks = 0; ks < K / 16; ++ks)
                    tc_mma(tmem, tc_desc(a_addr + ks * 256, 128, sbo),
                           tc_desc(w_addr + tc_w_offset(l) + ks * 256, 128, sbo), tc_idesc(TC_ROWS, N),
                           ks > 0 ? 1u : 0u);
                tc_commit(mb);
            }
            const bool done = mbar_wait(mb, phase);
            phase ^= 1u;
            tc_fence_after();
            if(!done)
                ;  // leave the accumulator unread; the group agrees on the timeout below
            else if(l + 1 < NRC_LAYERS)
            {
                unsigned char *dst = sa + tc_offset(erow, 0, NRC_WIDTH);
#pragma unroll 1
                for(int c = 0; c < NRC_WIDTH / 16; ++c)
                {
                    float v[16];
                    tc_ld16(tmem + lane_base + static_cast<uint32_t>(16 * c), v);
#pragma unroll
                    for(int h = 0; h < 2; ++h)
                        *reinterpret_cast<uint4 *>(dst + (2 * c + h) * 128) =
                            make_uint4(pack_bf16(fmaxf(v[8 * h + 0], 0.0f), fmaxf(v[8 * h + 1], 0.0f)),
                                       pack_bf16(fmaxf(v[8 * h + 2], 0.0f), fmaxf(v[8 * h + 3], 0.0f)),
                                       pack_bf16(fmaxf(v[8 * h + 4], 0.0f), fmaxf(v[8 * h + 5], 0.0f)),
                                       pack_bf16(fmaxf(v[8 * h + 6], 0.0f), fmaxf(v[8 * h + 7], 0.0f)));
                }
                fence_async_smem();
            }
            else
            {
                float v[4];
                tc_ld4(tmem + lane_base, v);
                const uint32_t r = tile * TC_ROWS + erow;
                if(r < n)
                    *reinterpret_cast<float4 *>(out + static_cast<size_t>(r) * 4) = make_float4(v[0], v[1], v[2], v[3]);
            }
            tc_fence_before();
            ok = group_sync_and(g, done);
        }
    }
    if(!ok && m == 0)
        atomicOr(D.err, 1u);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if(warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(*tmem_slot), "r"(TC_TMEM_COLS)
                     : "memory");
}

// ------------------------------------------------------------------ training: fused fwd + bwd

__global__ void __launch_bounds__(NRC_BLOCK) k_nrc_train(NrcDev D, const float *__restrict__ samples, uint32_t n,
                                                         float rel_eps)
{
    extern __shared__ uint4 smem_raw[];
    uint2 *swf = reinterpret_cast<uint2 *>(smem_raw);
    uint2 *swb = swf + FWD_PACKED;
    __nv_bfloat16 *sx = reinterpret_cast<__nv_bfloat16 *>(swb + BWD_PACKED);
    load_weights(D.w_fwd, swf, FWD_PACKED);
    load_weights(D.w_bwd, swb, BWD_PACKED);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    // per warp: X0 (16 x 88), X1..X5 (5 x 16 x 72) bf16, then 16 x 32 floats for dX0 and
    // 16 x 4 floats for the targets
    const int warp_elems = 16 * X0_STRIDE + (NRC_LAYERS - 1) * 16 * XH_STRIDE;
    __nv_bfloat16 *x0 = sx + warp * warp_elems;
    __nv_bfloat16 *xh = x0 + 16 * X0_STRIDE;
    float *sdx = reinterpret_cast<float *>(sx + NRC_WARPS * warp_elems) + warp * (16 * 32 + 16 * 4);
    float *stgt = sdx + 16 * 32;
    const float inv_n = 1.0f / static_cast<float>(n);
    float loss_acc = 0.0f;
    const uint32_t tiles = (n + 15) / 16;
    for(uint32_t tile = blockIdx.x * NRC_WARPS + warp; tile < tiles; tile += gridDim.x * NRC_WARPS)
    {
        const uint32_t row = tile * 16 + (lane & 15);
        const bool valid = row < n;
        float q[NRC_SAMPLE_FLOATS];
        if(valid)
            for(int k = 0; k < NRC_SAMPLE_FLOATS; ++k)
                q[k] = samples[static_cast<size_t>(row) * NRC_SAMPLE_FLOATS + k];
        else
            for(int k = 0; k < NRC_SAMPLE_FLOATS; ++k)
                q[k] = k == 5 || k == 8 ? 1.0f : 0.0f;
        encode_half(D, q, lane >> 4, x0 + (lane & 15) * X0_STRIDE);
        if(lane < 16)
        {
            stgt[lane * 4 + 0] = q[13];
            stgt[lane * 4 + 1] = q[14];
            stgt[lane * 4 + 2] = q[15];
            stgt[lane * 4 + 3] = valid ? 1.0f : 0.0f;
        }
        __syncwarp();
        // ---- forward, keeping each layer's input in shared memory
        uint32_t a[4][4];
        {
            float acc[8][4];
#pragma unroll
            for(int nt = 0; nt < 8; ++nt)
                acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
            for(int kt = 0; kt < 5; ++kt)
            {
                uint32_t ax[4];
                load_a(x0, X0_STRIDE, kt, lane, ax);
#pragma unroll
                for(int nt = 0; nt < 8; ++nt)
                    mma(acc[nt], ax, swf[(kt * 8 + nt) * 32 + lane]);
            }
#pragma unroll
            for(int kt = 0; kt < 4; ++kt)
            {
                acc_to_a_relu(acc[2 * kt], acc[2 * kt + 1], a[kt]);
                store_a(xh, XH_STRIDE, kt, lane, a[kt]);
            }
        }
#pragma unroll 1
        for(int l = 1; l < NRC_LAYERS - 1; ++l)
        {
            hidden_layer(swf, l, lane, a);
#pragma unroll
            for(int kt = 0; kt < 4; ++kt)
                store_a(xh + l * 16 * XH_STRIDE, XH_STRIDE, kt, lane, a[kt]);
        }
        float o[2][4] = { { 0, 0, 0, 0 }, { 0, 0, 0, 0 } };
        {
            const uint2 *w5 = swf + fwd_base(NRC_LAYERS - 1);
#pragma unroll
            for(int kt = 0; kt < 4; ++kt)
            {
                mma(o[0], a[kt], w5[(kt * 2 + 0) * 32 + lane]);
                mma(o[1], a[kt], w5[(kt * 2 + 1) * 32 + lane]);
            }
        }
        __syncwarp();
        // ---- relative L2 loss on outputs 0..2 and its gradient dY5 (16 x 16)
        float dy5[2][4] = { { 0, 0, 0, 0 }, { 0, 0, 0, 0 } };
#pragma unroll
        for(int h = 0; h < 2; ++h)
        {
            const int r = g + 8 * h;
            const float vrow = stgt[r * 4 + 3];
#pragma unroll
            for(int j = 0; j < 2; ++j)
            {
                const int col = 2 * t + j;
                if(col < 3 && vrow != 0.0f)
                {
                    const float y = o[0][2 * h + j], tg = stgt[r * 4 + col];
                    const float den = 1.0f / (y * y + rel_eps);
                    const float diff = y - tg;
                    loss_acc += diff * diff * den * inv_n;
                    dy5[0][2 * h + j] = 2.0f * diff * den * inv_n;
                }
            }
        }
        // ---- backward: dX = dY W^T, dY_prev = dX * (X > 0)
        uint32_t da[4][4];
        da[0][0] = pack_bf16(dy5[0][0], dy5[0][1]);
        da[0][1] = pack_bf16(dy5[0][2], dy5[0][3]);
        da[0][2] = pack_bf16(dy5[1][0], dy5[1][1]);
        da[0][3] = pack_bf16(dy5[1][2], dy5[1][3]);
        const size_t rbase = static_cast<size_t>(tile) * 16;
        // store dY5 rows (16 columns) and the layer inputs for the weight gradients
        {
            __nv_bfloat16 *dst = D.dact + rbase * DACT_COLS;
            uint32_t *r0 = reinterpret_cast<uint32_t *>(dst + g * DACT_COLS + dact_cols_before(5) + 2 * t);
            uint32_t *r1 = reinterpret_cast<uint32_t *>(dst + (g + 8) * DACT_COLS + dact_cols_before(5) + 2 * t);
            r0[0] = da[0][0];
            r1[0] = da[0][1];
            r0[4] = da[0][2];
            r1[4] = da[0][3];
        }
        for(int i = lane; i < 16 * (NRC_IN / 2); i += 32)
        {
            const int r = i / (NRC_IN / 2), c = (i % (NRC_IN / 2)) * 2;
            *reinterpret_cast<uint32_t *>(D.act + (rbase + r) * ACT_COLS + c) =
                *reinterpret_cast<const uint32_t *>(x0 + r * X0_STRIDE + c);
        }
        for(int l = 1; l < NRC_LAYERS; ++l)
            for(int i = lane; i < 16 * (NRC_WIDTH / 2); i += 32)
            {
                const int r = i / (NRC_WIDTH / 2), c = (i % (NRC_WIDTH / 2)) * 2;
                *reinterpret_cast<uint32_t *>(D.act + (rbase + r) * ACT_COLS + act_cols_before(l) + c) =
                    *reinterpret_cast<const uint32_t *>(xh + (l - 1) * 16 * XH_STRIDE + r * XH_STRIDE + c);
            }
        // layer 5: dX5 = dY5 W5^T (k' = 16 outputs, one k-tile), 64 columns
#pragma unroll 1
        for(int l = NRC_LAYERS - 1; l >= 1; --l)
        {
            const int kts = layer_n(l) / 16;          // k-tiles of dY_l
            const uint2 *wb = swb + bwd_base(l);
            float acc[8][4];
#pragma unroll
            for(int nt = 0; nt < 8; ++nt)
                acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
            for(int kt = 0; kt < 4; ++kt)
                if(kt < kts)
#pragma unroll
                    for(int nt = 0; nt < 8; ++nt)
                        mma(acc[nt], da[kt], wb[(kt * 8 + nt) * 32 + lane]);
            // ReLU derivative from X_l (the input of layer l = relu(Y_{l-1}))
            const __nv_bfloat16 *xl = xh + (l - 1) * 16 * XH_STRIDE;
#pragma unroll
            for(int nt = 0; nt < 8; ++nt)
            {
                const float2 m0 = unpack_bf16(*reinterpret_cast<const uint32_t *>(xl + g * XH_STRIDE + nt * 8 + 2 * t));
                const float2 m1 = unpack_bf16(*reinterpret_cast<const uint32_t *>(xl + (g + 8) * XH_STRIDE + nt * 8 + 2 * t));
                acc[nt][0] = m0.x > 0.0f ? acc[nt][0] : 0.0f;
                acc[nt][1] = m0.y > 0.0f ? acc[nt][1] : 0.0f;
                acc[nt][2] = m1.x > 0.0f ? acc[nt][2] : 0.0f;
                acc[nt][3] = m1.y > 0.0f ? acc[nt][3] : 0.0f;
            }
            // dY_{l-1} as A fragments; stored for dW_{l-1}
            __nv_bfloat16 *dst = D.dact + rbase * DACT_COLS + dact_cols_before(l - 1);
#pragma unroll
            for(int kt = 0; kt < 4; ++kt)
            {
                da[kt][0] = pack_bf16(acc[2 * kt][0], acc[2 * kt][1]);
                da[kt][1] = pack_bf16(acc[2 * kt][2], acc[2 * kt][3]);
                da[kt][2] = pack_bf16(acc[2 * kt + 1][0], acc[2 * kt + 1][1]);
                da[kt][3] = pack_bf16(acc[2 * kt + 1][2], acc[2 * kt + 1][3]);
                uint32_t *r0 = reinterpret_cast<uint32_t *>(dst + g * DACT_COLS + kt * 16 + 2 * t);
                uint32_t *r1 = reinterpret_cast<uint32_t *>(dst + (g + 8) * DACT_COLS + kt * 16 + 2 * t);
                r0[0] = da[kt][0];
                r1[0] = da[kt][1];
                r0[4] = da[kt][2];
                r1[4] = da[kt][3];
            }
        }
        // layer 0: dX0 (hash columns 0..31) = dY0 W0^T
        {
            const uint2 *wb = swb + bwd_base(0);
            float acc[4][4];
#pragma unroll
            for(int nt = 0; nt < 4; ++nt)
                acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
            for(int kt = 0; kt < 4; ++kt)
#pragma unroll
                for(int nt = 0; nt < 4; ++nt)
                    mma(acc[nt], da[kt], wb[(kt * 4 + nt) * 32 + lane]);
#pragma unroll
            for(int nt = 0; nt < 4; ++nt)
            {
                sdx[g * 32 + nt * 8 + 2 * t] = acc[nt][0];
                sdx[g * 32 + nt * 8 + 2 * t + 1] = acc[nt][1];
                sdx[(g + 8) * 32 + nt * 8 + 2 * t] = acc[nt][2];
                sdx[(g + 8) * 32 + nt * 8 + 2 * t + 1] = acc[nt][3];
            }
        }
        __syncwarp();
        // hash-table gradient: trilinear weights times dL/dfeature
        if(valid)
        {
            const int r = lane & 15, half = lane >> 4;
            const V3 p = nrc_unit_pos(D, q);
            for(int l = half * 8; l < half * 8 + 8; ++l)
            {
                uint32_t idx[8];
                float w[8];
                level_corners(p, l, idx, w);
                const float d0 = sdx[r * 32 + l * 2], d1 = sdx[r * 32 + l * 2 + 1];
#pragma unroll
                for(int c = 0; c < 8; ++c)
                    atomicAdd(D.hash_grad + idx[c], make_float2(w[c] * d0, w[c] * d1));
            }
        }
        __syncwarp();
    }
    // loss
    for(int off = 16; off > 0; off >>= 1)
        loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, off);
    if(lane == 0)
        atomicAdd(D.loss, loss_acc);
}

// ------------------------------------------------------------------ weight gradients

// dW_l[K][N] += X_l^T dY_l over 128 rows per block, for all layers at once (blockIdx.y =
// layer), on the tensor cores: A = X^T (K x rows), B = dY (rows x N). Rows are staged
// transposed in shared memory (an odd word stride keeps the transposing stores free of
// bank conflicts) so that fragments load as 32-bit pairs; every warp owns up to five
// 16 x 8 output tiles and adds them to the FP32 gradient with atomics.
constexpr int WG_ROWS = 128;
constexpr int WG_BLOCK = 256;
constexpr int WG_STRIDE = WG_ROWS + 2;    // 65 words per staged row

__global__ void __launch_bounds__(WG_BLOCK) k_nrc_wgrad(const __nv_bfloat16 *__restrict__ act,
                                                        const __nv_bfloat16 *__restrict__ dact, uint32_t n,
                                                        float *__restrict__ dw_all)
{
    __shared__ __nv_bfloat16 sxt[NRC_IN][WG_STRIDE];
    __shared__ __nv_bfloat16 sdt[NRC_WIDTH][WG_STRIDE];
    const int l = blockIdx.y;
    const int K = layer_k(l), N = layer_n(l);
    const int ntiles = N / 8, tiles = (K / 16) * ntiles;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = WG_BLOCK / 32;
    const int g = lane >> 2, t = lane & 3;
    constexpr int MAXT = 5;                    // at most 40 tiles over 8 warps
    float acc[MAXT][4];
#pragma unroll
    for(int i = 0; i < MAXT; ++i)
        acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.0f;
    const uint32_t r0 = blockIdx.x * WG_ROWS;
    const int acol = act_cols_before(l), dcol = dact_cols_before(l);
    // stage: consecutive threads read consecutive columns of a row (coalesced) and store
    // them down a column of the transposed tile
    for(int i = threadIdx.x; i < WG_ROWS * K; i += WG_BLOCK)
    {
        const int r = i / K, k = i % K;
        const uint32_t row = r0 + r;
        sxt[k][r] = row < n ? act[static_cast<size_t>(row) * ACT_COLS + acol + k] : __float2bfloat16_rn(0.0f);
    }
    for(int i = threadIdx.x; i < WG_ROWS * N; i += WG_BLOCK)
    {
        const int r = i / N, c = i % N;
        const uint32_t row = r0 + r;
        sdt[c][r] = row < n ? dact[static_cast<size_t>(row) * DACT_COLS + dcol + c] : __float2bfloat16_rn(0.0f);
    }
    __syncthreads();
#pragma unroll
    for(int slot = 0; slot < MAXT; ++slot)
    {
        const int tile = warp + slot * nwarps;
        if(tile >= tiles)
            break;
        const int mt = tile / ntiles, nt = tile % ntiles;
#pragma unroll 4
        for(int kk = 0; kk < WG_ROWS / 16; ++kk)
        {
            uint32_t a[4];
            const __nv_bfloat16 *ar0 = &sxt[mt * 16 + g][kk * 16 + 2 * t];
            const __nv_bfloat16 *ar1 = &sxt[mt * 16 + g + 8][kk * 16 + 2 * t];
            a[0] = *reinterpret_cast<const uint32_t *>(ar0);
            a[1] = *reinterpret_cast<const uint32_t *>(ar1);
            a[2] = *reinterpret_cast<const uint32_t *>(ar0 + 8);
            a[3] = *reinterpret_cast<const uint32_t *>(ar1 + 8);
            const __nv_bfloat16 *br = &sdt[nt * 8 + g][kk * 16 + 2 * t];
            uint2 b;
            b.x = *reinterpret_cast<const uint32_t *>(br);
            b.y = *reinterpret_cast<const uint32_t *>(br + 8);
            mma(acc[slot], a, b);
        }
    }
    float *dw = dw_all + w_offset(l);
#pragma unroll
    for(int slot = 0; slot < MAXT; ++slot)
    {
        const int tile = warp + slot * nwarps;
        if(tile >= tiles)
            break;
        const int mt = tile / ntiles, nt = tile % ntiles;
        const int r = mt * 16 + g, c = nt * 8 + 2 * t;
        atomicAdd(dw + r * N + c, acc[slot][0]);
        atomicAdd(dw + r * N + c + 1, acc[slot][1]);
        atomicAdd(dw + (r + 8) * N + c, acc[slot][2]);
        atomicAdd(dw + (r + 8) * N + c + 1, acc[slot][3]);
    }
}

// ------------------------------------------------------------------ Adam and packing

__global__ void k_nrc_adam(float *__restrict__ p, float *__restrict__ grad, float *__restrict__ m,
                           float *__restrict__ v, uint64_t count, float lr_t, float b1, float b2, float eps)
{
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for(uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < count; i += stride)
    {
        const float gr = grad[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gr;
        const float vi = b2 * v[i] + (1.0f - b2) * gr * gr;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr_t * mi / (sqrtf(vi) + eps);
        grad[i] = 0.0f;
    }
}

__global__ void k_nrc_hash_to_f16(const float2 *__restrict__ src, __half2 *__restrict__ dst, uint64_t count)
{
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for(uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < count; i += stride)
        dst[i] = __floats2half2_rn(src[i].x, src[i].y);
}

__global__ void k_nrc_pack(const float *__restrict__ w, uint2 *__restrict__ fwd, uint2 *__restrict__ bwd,
                           __nv_bfloat16 *__restrict__ wtc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < NRC_WEIGHTS)
    {
        // W_l (row-major K x N) -> W_l^T as an N x K K-major operand in core matrices
        int l = 0;
        while(l + 1 < NRC_LAYERS && i >= w_offset(l + 1))
            ++l;
        const int local = i - w_offset(l), N = layer_n(l), K = layer_k(l);
        const int k = local / N, c = local % N;
        wtc[(tc_w_offset(l) + tc_offset(c, k, K)) / 2] = __float2bfloat16_rn(w[i]);
    }
    if(i < FWD_PACKED)
    {
        int l = 0;
        while(l + 1 < NRC_LAYERS && i >= fwd_base(l + 1))
            ++l;
        const int local = i - fwd_base(l), lane = local % 32, tile = local / 32;
        const int N = layer_n(l), nts = N / 8, kt = tile / nts, nt = tile % nts;
        const int g = lane >> 2, t = lane & 3;
        const float *W = w + w_offset(l);
        const int k0 = kt * 16 + 2 * t, c = nt * 8 + g;
        fwd[i] = make_uint2(pack_bf16(W[k0 * N + c], W[(k0 + 1) * N + c]),
                            pack_bf16(W[(k0 + 8) * N + c], W[(k0 + 9) * N + c]));
    }
    if(i < BWD_PACKED)
    {
        int l = 0;
        while(l + 1 < NRC_LAYERS && i >= bwd_base(l + 1))
            ++l;
        const int local = i - bwd_base(l), lane = local % 32, tile = local / 32;
        const int N = layer_n(l), nts = bwd_n(l) / 8, kt = tile / nts, nt = tile % nts;
        const int g = lane >> 2, t = lane & 3;
        const float *W = w + w_offset(l);
        // B' = W^T: B'[k'][n'] = W[n'][k'], k' over the N outputs, n' over the inputs
        const int k0 = kt * 16 + 2 * t, r = nt * 8 + g;
        bwd[i] = make_uint2(pack_bf16(W[r * N + k0], W[r * N + k0 + 1]), pack_bf16(W[r * N + k0 + 8], W[r * N + k0 + 9]));
    }
}

size_t infer_smem() { return FWD_PACKED * sizeof(uint2) + NRC_WARPS * 16 * X0_STRIDE * sizeof(__nv_bfloat16); }
size_t infer_tc_smem() { return TC_W_BYTES + TC_GROUPS * TC_A_BYTES + 8 * TC_GROUPS + 16; }
size_t train_smem()
{
    return (FWD_PACKED + BWD_PACKED) * sizeof(uint2) +
           NRC_WARPS * (16 * X0_STRIDE + (NRC_LAYERS - 1) * 16 * XH_STRIDE) * sizeof(__nv_bfloat16) +
           NRC_WARPS * (16 * 32 + 16 * 4) * sizeof(float);
}

int sm_count()
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

// SplitMix64 for parameter initialisation
uint64_t splitmix(uint64_t &s)
{
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
float uniform01(uint64_t &s) { return static_cast<float>(splitmix(s) >> 40) * (1.0f / 16777216.0f); }

} // namespace

#define NRC_CHECK(x)                                                                                                  \
    do                                                                                                                \
    {                                                                                                                 \
        cudaError_t e_ = (x);                                                                                         \
        if(e_ != cudaSuccess)                                                                                         \
            return e_;                                                                                                \
    } while(0)

Nrc::Nrc(const float bbox_min[3], const float bbox_max[3], uint64_t seed)
{
    for(int a = 0; a < 3; ++a)
    {
        const float ext = bbox_max[a] - bbox_min[a];
        d_.bbox_min[a] = bbox_min[a] - 1e-3f * ext;
        d_.bbox_inv_extent[a] = ext > 0 ? 1.0f / (ext * 1.002f) : 1.0f;
    }
    // level resolutions N_l = N_min b^l, dense storage where the grid fits the table
    LevelInfo levels[NRC_LEVELS];
    const double b = std::exp((std::log(NRC_MAX_RES) - std::log(NRC_MIN_RES)) / (NRC_LEVELS - 1));
    for(int l = 0; l < NRC_LEVELS; ++l)
    {
        levels[l].res = static_cast<float>(std::floor(NRC_MIN_RES * std::pow(b, l)));
        const uint64_t s = static_cast<uint64_t>(levels[l].res) + 2;
        levels[l].stride = s * s * s <= NRC_TABLE ? static_cast<uint32_t>(s) : 0u;
    }
    auto fail = [](cudaError_t e) {
        if(e != cudaSuccess)
            throw std::runtime_error(std::string("radiance cache: ") + cudaGetErrorString(e));
    };
    fail(cudaMemcpyToSymbol(c_levels, levels, sizeof(levels)));
    const uint64_t hcount = static_cast<uint64_t>(NRC_LEVELS) * NRC_TABLE;
    fail(cudaMalloc(&w_master_, sizeof(float) * NRC_WEIGHTS));
    fail(cudaMalloc(&w_grad_, sizeof(float) * NRC_WEIGHTS));
    fail(cudaMalloc(&w_m_, sizeof(float) * NRC_WEIGHTS));
    fail(cudaMalloc(&w_v_, sizeof(float) * NRC_WEIGHTS));
    fail(cudaMalloc(&h_master_, sizeof(float2) * hcount));
    fail(cudaMalloc(&h_m_, sizeof(float2) * hcount));
    fail(cudaMalloc(&h_v_, sizeof(float2) * hcount));
    fail(cudaMalloc(&d_.hash_grad, sizeof(float2) * hcount));
    fail(cudaMalloc(&h_f16_, sizeof(__half2) * hcount));
    fail(cudaMalloc(&w_fwd_, sizeof(uint2) * FWD_PACKED));
    fail(cudaMalloc(&w_bwd_, sizeof(uint2) * BWD_PACKED));
    fail(cudaMalloc(&w_tc_, TC_W_BYTES));
    fail(cudaMalloc(&err_, sizeof(uint32_t)));
    fail(cudaMemset(err_, 0, sizeof(uint32_t)));
    fail(cudaMalloc(&loss_, sizeof(float)));
    fail(cudaMemset(w_grad_, 0, sizeof(float) * NRC_WEIGHTS));
    fail(cudaMemset(w_m_, 0, sizeof(float) * NRC_WEIGHTS));
    fail(cudaMemset(w_v_, 0, sizeof(float) * NRC_WEIGHTS));
    fail(cudaMemset(h_m_, 0, sizeof(float2) * hcount));
    fail(cudaMemset(h_v_, 0, sizeof(float2) * hcount));
    fail(cudaMemset(d_.hash_grad, 0, sizeof(float2) * hcount));
    // initialisation: uniform +-sqrt(6 / (fan_in + fan_out)) weights, zero padded output
    // columns, hash features uniform in +-1e-4
    uint64_t s = seed;
    std::vector<float> w(NRC_WEIGHTS);
    for(int l = 0; l < NRC_LAYERS; ++l)
    {
        const int K = layer_k(l), N = layer_n(l);
        const int fan_out = l == NRC_LAYERS - 1 ? 3 : N;
        const float lim = std::sqrt(6.0f / static_cast<float>(K + fan_out));
        for(int k = 0; k < K; ++k)
            for(int c = 0; c < N; ++c)
                w[w_offset(l) + k * N + c] = (l == NRC_LAYERS - 1 && c >= 3) ? 0.0f : (2.0f * uniform01(s) - 1.0f) * lim;
    }
    fail(cudaMemcpy(w_master_, w.data(), sizeof(float) * NRC_WEIGHTS, cudaMemcpyHostToDevice));
    std::vector<float> h(hcount * 2);
    for(float &x : h)
        x = (2.0f * uniform01(s) - 1.0f) * 1e-4f;
    fail(cudaMemcpy(h_master_, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice));
    d_.hash = h_f16_;
    d_.w_fwd = w_fwd_;
    d_.w_bwd = w_bwd_;
    d_.w_tc = w_tc_;
    d_.err = err_;
    d_.loss = loss_;
    fail(cudaFuncSetAttribute(k_nrc_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(infer_smem())));
    fail(cudaFuncSetAttribute(k_nrc_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(infer_tc_smem())));
    fail(cudaFuncSetAttribute(k_nrc_train, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(train_smem())));
    // inference kernel: tcgen05 (default) or the mma.sync kernel (BTRC_NRC_INFER=mma)
    if(const char *k = std::getenv("BTRC_NRC_INFER"))
        use_tc_ = std::strcmp(k, "mma") != 0;
    fail(repack(nullptr));
    fail(cudaStreamSynchronize(nullptr));
}

Nrc::~Nrc()
{
    for(void *p : { static_cast<void *>(w_master_), static_cast<void *>(w_grad_), static_cast<void *>(w_m_),
                    static_cast<void *>(w_v_), static_cast<void *>(h_master_), static_cast<void *>(h_m_),
                    static_cast<void *>(h_v_), static_cast<void *>(d_.hash_grad), static_cast<void *>(h_f16_),
                    static_cast<void *>(w_fwd_), static_cast<void *>(w_bwd_), static_cast<void *>(loss_),
                    static_cast<void *>(w_tc_), static_cast<void *>(err_),
                    static_cast<void *>(act_), static_cast<void *>(dact_) })
        if(p)
            cudaFree(p);
}

cudaError_t Nrc::repack(cudaStream_t st)
{
    const int n = std::max(NRC_WEIGHTS, std::max(FWD_PACKED, BWD_PACKED));
    k_nrc_pack<<<(n + 255) / 256, 256, 0, st>>>(w_master_, w_fwd_, w_bwd_, w_tc_);
    NRC_CHECK(cudaGetLastError());
    const uint64_t hcount = static_cast<uint64_t>(NRC_LEVELS) * NRC_TABLE;
    k_nrc_hash_to_f16<<<sm_count() * 8, 256, 0, st>>>(h_master_, h_f16_, hcount);
    return cudaGetLastError();
}

cudaError_t Nrc::ensure_batch(uint32_t n)
{
    if(n <= batch_cap_)
        return cudaSuccess;
    if(act_)
        cudaFree(act_);
    if(dact_)
        cudaFree(dact_);
    act_ = dact_ = nullptr;
    batch_cap_ = 0;
    const uint32_t cap = (n + 15) / 16 * 16;
    NRC_CHECK(cudaMalloc(&act_, sizeof(__nv_bfloat16) * static_cast<size_t>(cap) * ACT_COLS));
    NRC_CHECK(cudaMalloc(&dact_, sizeof(__nv_bfloat16) * static_cast<size_t>(cap) * DACT_COLS));
    d_.act = act_;
    d_.dact = dact_;
    batch_cap_ = cap;
    return cudaSuccess;
}

cudaError_t Nrc::infer(const float *d_queries, uint32_t n, float *d_out, cudaStream_t st)
{
    if(n == 0)
        return cudaSuccess;
    if(use_tc_)
    {
        const uint32_t tiles = (n + TC_ROWS - 1) / TC_ROWS;
        const uint32_t blocks = std::min<uint32_t>((tiles + TC_GROUPS - 1) / TC_GROUPS, static_cast<uint32_t>(sm_count()));
        k_nrc_infer_tc<<<blocks, TC_BLOCK, infer_tc_smem(), st>>>(d_, d_queries, n, d_out);
        return cudaGetLastError();
    }
    const uint32_t tiles = (n + 15) / 16;
    const uint32_t blocks = std::min<uint32_t>((tiles + NRC_WARPS - 1) / NRC_WARPS, static_cast<uint32_t>(sm_count()) * 8);
    k_nrc_infer<<<blocks, NRC_BLOCK, infer_smem(), st>>>(d_, d_queries, n, d_out);
    return cudaGetLastError();
}

cudaError_t Nrc::reset_loss(cudaStream_t st) { return cudaMemsetAsync(loss_, 0, sizeof(float), st); }

cudaError_t Nrc::read_loss(float *out, cudaStream_t st)
{
    NRC_CHECK(cudaMemcpyAsync(out, loss_, sizeof(float), cudaMemcpyDeviceToHost, st));
    NRC_CHECK(cudaStreamSynchronize(st));
    return check_error(st);
}

cudaError_t Nrc::copy_loss_async(float *out, cudaStream_t st)
{
    return cudaMemcpyAsync(out, loss_, sizeof(float), cudaMemcpyDeviceToHost, st);
}

cudaError_t Nrc::check_error(cudaStream_t st)
{
    uint32_t e = 0;
    NRC_CHECK(cudaMemcpyAsync(&e, err_, sizeof(e), cudaMemcpyDeviceToHost, st));
    NRC_CHECK(cudaStreamSynchronize(st));
    return e ? cudaErrorLaunchTimeout : cudaSuccess;
}

cudaError_t Nrc::train(const float *d_samples, uint32_t n, bool apply_adam, cudaStream_t st)
{
    if(n == 0)
        return cudaSuccess;
    NRC_CHECK(ensure_batch(n));
    const uint32_t tiles = (n + 15) / 16;
    const uint32_t blocks = std::min<uint32_t>((tiles + NRC_WARPS - 1) / NRC_WARPS, static_cast<uint32_t>(sm_count()) * 4);
    k_nrc_train<<<blocks, NRC_BLOCK, train_smem(), st>>>(d_, d_samples, n, hyper_.rel_eps);
    NRC_CHECK(cudaGetLastError());
    k_nrc_wgrad<<<dim3((n + WG_ROWS - 1) / WG_ROWS, NRC_LAYERS), WG_BLOCK, 0, st>>>(act_, dact_, n, w_grad_);
    NRC_CHECK(cudaGetLastError());
    if(apply_adam)
    {
        ++step_;
        const float bc1 = 1.0f - std::pow(hyper_.beta1, static_cast<float>(step_));
        const float bc2 = 1.0f - std::pow(hyper_.beta2, static_cast<float>(step_));
        const float lr_t = hyper_.lr * std::sqrt(bc2) / bc1;
        k_nrc_adam<<<(NRC_WEIGHTS + 255) / 256, 256, 0, st>>>(w_master_, w_grad_, w_m_, w_v_, NRC_WEIGHTS, lr_t,
                                                             hyper_.beta1, hyper_.beta2, hyper_.eps);
        NRC_CHECK(cudaGetLastError());
        const uint64_t hcount = static_cast<uint64_t>(NRC_LEVELS) * NRC_TABLE * 2;
        k_nrc_adam<<<sm_count() * 8, 256, 0, st>>>(reinterpret_cast<float *>(h_master_),
                                                   reinterpret_cast<float *>(d_.hash_grad),
                                                   reinterpret_cast<float *>(h_m_), reinterpret_cast<float *>(h_v_),
                                                   hcount, lr_t, hyper_.beta1, hyper_.beta2, hyper_.eps);
        NRC_CHECK(cudaGetLastError());
        NRC_CHECK(repack(st));
    }
    return cudaSuccess;
}

cudaError_t Nrc::copy_params(int which, float *host, uint64_t count, bool set, cudaStream_t st)
{
    const uint64_t hcount = static_cast<uint64_t>(NRC_LEVELS) * NRC_TABLE * 2;
    float *src = nullptr;
    uint64_t n = 0;
    switch(which)
    {
    case 0: src = w_master_; n = NRC_WEIGHTS; break;
    case 1: src = reinterpret_cast<float *>(h_master_); n = hcount; break;
    case 2: src = w_grad_; n = NRC_WEIGHTS; break;
    case 3: src = reinterpret_cast<float *>(d_.hash_grad); n = hcount; break;
    default: return cudaErrorInvalidValue;
    }
    if(count != n)
        return cudaErrorInvalidValue;
    if(set)
    {
        NRC_CHECK(cudaMemcpyAsync(src, host, sizeof(float) * n, cudaMemcpyHostToDevice, st));
        if(which <= 1)
            NRC_CHECK(repack(st));
    }
    else
        NRC_CHECK(cudaMemcpyAsync(host, src, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    NRC_CHECK(cudaStreamSynchronize(st));
    return check_error(st);
}

} // namespace bt
