// manet.cu -- the Monge-Ampere warm-start network: 4 periodic 3x3x3 convolutions
// (3 -> 16 -> 16 -> 16 -> 1 channels, ReLU after the first three) on BF16 tensor cores with FP32
// accumulation, forward, backward and Adam, all on the device.
//
// Tensors are channel-last BF16 [N^3][16] (32 bytes per voxel; the 3-channel input and the
// 1-channel output are zero padded to 16, so every layer is one kernel shape).  Voxel
// v = (x N + y) N + z, tap t = (dx+1) 9 + (dy+1) 3 + (dz+1):
//   out[v][co] = b[co] + sum_t sum_ci in[v + d_t][ci] w[t][ci][co]          (periodic)
//
// A convolution is an implicit GEMM per brick of 4 x 8 x 32 outputs: the brick and a one-voxel
// halo are staged in shared memory, each warp owns eight 16-voxel z-runs (M = 16 rows of the
// mma), and for every tap the 16 x 16 (voxel x channel) A tile is a shifted window of the staged
// brick loaded with ldmatrix; the 16 x 16 weight tile of the tap is the B operand.  Voxel rows are
// 32 bytes; their two 16-byte halves are XOR-swizzled by bit 2 of the voxel index so that the
// eight rows of any ldmatrix phase hit distinct banks.
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "context.cuh"

namespace mitos {

#define MN_C 16                 // stored channels
#define MN_BX 4                 // brick of outputs
#define MN_BY 8
#define MN_BZ 32
#define MN_TX (MN_BX + 2)       // staged tile (brick + halo)
#define MN_TY (MN_BY + 2)
#define MN_TZ (MN_BZ + 2)
#define MN_THREADS 256          // 8 warps x 8 m-tiles
#define MN_TILE_VOX (MN_TX * MN_TY * MN_TZ)
#define MN_BRICK_VOX (MN_BX * MN_BY * MN_BZ)
#define MN_WPL (27 * MN_C * MN_C)          // weights per layer (padded)
#define MN_PPL (MN_WPL + MN_C)             // parameters per layer: weights + biases

static_assert(MANET_PARAMS == 4 * MN_PPL, "parameter count");

// ---- small PTX helpers ---------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}
// D = A (16x16 bf16, row) * B (16x8 bf16, col) + D, FP32 accumulators
__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ void cp16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// byte offset of the 16-byte half h of 32-byte row r in a swizzled staging array
__device__ __forceinline__ int swz(int r, int h) { return r * 32 + ((h ^ ((r >> 2) & 1)) << 4); }

__device__ __forceinline__ int wrapc(int i, int N) { return i < 0 ? i + N : (i >= N ? i - N : i); }

// stage the brick's input tile (with a one-voxel periodic halo) and one layer's 27 weight tiles
__device__ __forceinline__ void stage_tile(unsigned char *tile, const __nv_bfloat16 *__restrict__ in, int N, int x0,
                                           int y0, int z0) {
    for (int c = threadIdx.x; c < MN_TILE_VOX * 2; c += MN_THREADS) {
        const int v = c >> 1, h = c & 1;
        const int tz = v % MN_TZ, ty = (v / MN_TZ) % MN_TY, tx = v / (MN_TZ * MN_TY);
        const long gv = ((long)wrapc(x0 + tx - 1, N) * N + wrapc(y0 + ty - 1, N)) * N + wrapc(z0 + tz - 1, N);
        cp16(tile + swz(v, h), in + gv * MN_C + h * 8);
    }
}
__device__ __forceinline__ void stage_weights(unsigned char *wsm, const __nv_bfloat16 *__restrict__ w) {
    // 27 taps x 16 rows (n) x 2 halves (k)
    for (int c = threadIdx.x; c < 27 * MN_C * 2; c += MN_THREADS) {
        const int r = c >> 1, h = c & 1;  // r = tap * 16 + n
        cp16(wsm + swz(r, h), w + r * MN_C + h * 8);
    }
}

__device__ __forceinline__ void brick_origin(int N, int &x0, int &y0, int &z0) {
    const int nbz = N / MN_BZ, nby = N / MN_BY;
    const int b = blockIdx.x;
    z0 = (b % nbz) * MN_BZ;
    y0 = ((b / nbz) % nby) * MN_BY;
    x0 = (b / (nbz * nby)) * MN_BX;
}

enum ConvMode { CONV_RELU = 0, CONV_LINEAR_OUT = 1, CONV_BWD_MASK = 2 };

// One convolution layer.  w: BF16 [27][16 (n)][16 (k)] (the B operands, per tap).
//   CONV_RELU:       out = bf16(relu(conv + b))                     (hidden layers)
//   CONV_LINEAR_OUT: outf[(x N + y) pitch + z] = scale (conv + b)[0] (last layer, FP32 grid)
//   CONV_BWD_MASK:   out = bf16(conv * (mask > 0))                 (gradient w.r.t. a hidden
//                    activation; w holds the tap-mirrored, transposed weights)
template <int MODE>
__global__ void __launch_bounds__(MN_THREADS, 2)
k_conv(int N, const __nv_bfloat16 *__restrict__ in, const __nv_bfloat16 *__restrict__ w, const float *__restrict__ bias,
       const __nv_bfloat16 *__restrict__ mask, __nv_bfloat16 *__restrict__ out, float *__restrict__ outf, int pitch,
       float scale) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *tile = smem;                        // MN_TILE_VOX * 32 bytes
    unsigned char *wsm = smem + MN_TILE_VOX * 32;      // 27 * 16 * 32 bytes
    int x0, y0, z0;
    brick_origin(N, x0, y0, z0);
    stage_tile(tile, in, N, x0, y0, z0);
    stage_weights(wsm, w);
    cp_wait_all();
    __syncthreads();

    constexpr int NT = (MODE == CONV_LINEAR_OUT) ? 1 : 2;  // n-tiles of 8 output channels
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float acc[8][NT][4];
#pragma unroll
    for (int m = 0; m < 8; m++)
#pragma unroll
        for (int n = 0; n < NT; n++)
#pragma unroll
            for (int j = 0; j < 4; j++) acc[m][n][j] = 0.f;

    const uint32_t tile_s = smem_u32(tile), w_s = smem_u32(wsm);
    const int arow = lane & 15, ahalf = lane >> 4;            // A: row of the 16-voxel run, k half
    const int bn = ((lane >> 4) << 3) + (lane & 7), bh = (lane >> 3) & 1;  // B: n row, k half
#pragma unroll 1
    for (int t = 0; t < 27; t++) {
        const int dx = t / 9 - 1, dy = (t / 3) % 3 - 1, dz = t % 3 - 1;
        uint32_t b[2][2];
        ldsm_x4(w_s + swz(t * MN_C + bn, bh), b[0][0], b[0][1], b[1][0], b[1][1]);
#pragma unroll
        for (int m = 0; m < 8; m++) {
            const int row = warp * 4 + (m >> 1);               // (lx, ly) run of the brick
            const int lx = row / MN_BY, ly = row % MN_BY, zr = (m & 1) * 16;
            const int v = ((lx + 1 + dx) * MN_TY + (ly + 1 + dy)) * MN_TZ + zr + 1 + dz + arow;
            uint32_t a[4];
            ldsm_x4(tile_s + swz(v, ahalf), a[0], a[1], a[2], a[3]);
#pragma unroll
            for (int n = 0; n < NT; n++) mma_bf16(acc[m][n], a, b[n][0], b[n][1]);
        }
    }

    // epilogue: lane holds rows g, g + 8 and output channels n*8 + 2q, +1
    const int g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int m = 0; m < 8; m++) {
        const int row = warp * 4 + (m >> 1);
        const int x = x0 + row / MN_BY, y = y0 + row % MN_BY, zb = z0 + (m & 1) * 16;
#pragma unroll
        for (int hr = 0; hr < 2; hr++) {
            const int z = zb + g + hr * 8;
            const long gv = ((long)x * N + y) * N + z;
            if constexpr (MODE == CONV_LINEAR_OUT) {
                if (q == 0) outf[((long)x * N + y) * pitch + z] = scale * (acc[m][0][hr * 2] + bias[0]);
            } else {
#pragma unroll
                for (int n = 0; n < NT; n++) {
                    const int c = n * 8 + 2 * q;
                    float v0 = acc[m][n][hr * 2], v1 = acc[m][n][hr * 2 + 1];
                    if constexpr (MODE == CONV_RELU) {
                        v0 = fmaxf(v0 + bias[c], 0.f);
                        v1 = fmaxf(v1 + bias[c + 1], 0.f);
                    } else {
                        const __nv_bfloat162 mk2 = *reinterpret_cast<const __nv_bfloat162 *>(mask + gv * MN_C + c);
                        if (!(__bfloat162float(mk2.x) > 0.f)) v0 = 0.f;
                        if (!(__bfloat162float(mk2.y) > 0.f)) v1 = 0.f;
                    }
                    *reinterpret_cast<__nv_bfloat162 *>(out + gv * MN_C + c) = __floats2bfloat162_rn(v0, v1);
                }
            }
        }
    }
}

// Weight gradients of one layer over one brick:
//   part[blk][(t*16 + ci)*16 + co] = sum_{v in brick} in[v + d_t][ci] dout[v][co],
//   part[blk][MN_WPL + co]         = sum_{v in brick} dout[v][co].
// mma with M = ci, N = co, K = 16 voxels of a z-run; warp w owns taps w, w + 8, w + 16, w + 24.
__global__ void __launch_bounds__(MN_THREADS, 2)
k_conv_wgrad(int N, const __nv_bfloat16 *__restrict__ in, const __nv_bfloat16 *__restrict__ dout, float *__restrict__ part) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *tile = smem;                        // MN_TILE_VOX * 32 bytes
    unsigned char *gsm = smem + MN_TILE_VOX * 32;      // MN_BRICK_VOX * 32 bytes
    __shared__ float dbs[MN_THREADS];
    int x0, y0, z0;
    brick_origin(N, x0, y0, z0);
    stage_tile(tile, in, N, x0, y0, z0);
    for (int c = threadIdx.x; c < MN_BRICK_VOX * 2; c += MN_THREADS) {
        const int v = c >> 1, h = c & 1;
        const int bz = v % MN_BZ, by = (v / MN_BZ) % MN_BY, bx = v / (MN_BZ * MN_BY);
        const long gv = ((long)(x0 + bx) * N + y0 + by) * N + z0 + bz;
        cp16(gsm + swz(v, h), dout + gv * MN_C + h * 8);
    }
    cp_wait_all();
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float acc[4][2][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int n = 0; n < 2; n++)
#pragma unroll
            for (int j = 0; j < 4; j++) acc[i][n][j] = 0.f;
    const uint32_t tile_s = smem_u32(tile), g_s = smem_u32(gsm);
    const int lm = lane >> 3, lr = lane & 7;
    const int av = ((lm >> 1) << 3) + lr, ah = lm & 1;   // A^T: voxel row, ci half
    const int bv = ((lm & 1) << 3) + lr, bh = lm >> 1;   // B^T: voxel row, co half
    const int ntap = (warp < 3) ? 4 : 3;
#pragma unroll 1
    for (int kc = 0; kc < MN_BRICK_VOX / 16; kc++) {
        const int row = kc >> 1, zr = (kc & 1) * 16;
        const int lx = row / MN_BY, ly = row % MN_BY;
        uint32_t b[2][2];
        ldsm_x4_t(g_s + swz((lx * MN_BY + ly) * MN_BZ + zr + bv, bh), b[0][0], b[0][1], b[1][0], b[1][1]);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            if (i < ntap) {
                const int t = warp + 8 * i;
                const int dx = t / 9 - 1, dy = (t / 3) % 3 - 1, dz = t % 3 - 1;
                const int v = ((lx + 1 + dx) * MN_TY + (ly + 1 + dy)) * MN_TZ + zr + 1 + dz + av;
                uint32_t a[4];
                ldsm_x4_t(tile_s + swz(v, ah), a[0], a[1], a[2], a[3]);
                mma_bf16(acc[i][0], a, b[0][0], b[0][1]);
                mma_bf16(acc[i][1], a, b[1][0], b[1][1]);
            }
        }
    }
    float *dst = part + (long)blockIdx.x * MN_PPL;
    const int g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        if (i < ntap) {
            const int t = warp + 8 * i;
#pragma unroll
            for (int n = 0; n < 2; n++)
#pragma unroll
                for (int hr = 0; hr < 2; hr++) {
                    const int ci = g + hr * 8, co = n * 8 + 2 * q;
                    dst[(t * MN_C + ci) * MN_C + co] = acc[i][n][hr * 2];
                    dst[(t * MN_C + ci) * MN_C + co + 1] = acc[i][n][hr * 2 + 1];
                }
        }
    }
    // bias gradient: thread k sums channel k % 16 over voxels k / 16, k / 16 + 16, ...
    {
        const int co = threadIdx.x & 15;
        float s = 0.f;
        for (int v = threadIdx.x >> 4; v < MN_BRICK_VOX; v += MN_THREADS / 16) {
            const int h = co >> 3;
            const __nv_bfloat16 *p = reinterpret_cast<const __nv_bfloat16 *>(gsm + swz(v, h));
            s += __bfloat162float(p[co & 7]);
        }
        dbs[threadIdx.x] = s;
        __syncthreads();
        if (threadIdx.x < MN_C) {
            float t = 0.f;
            for (int k = threadIdx.x; k < MN_THREADS; k += MN_C) t += dbs[k];
            dst[MN_WPL + threadIdx.x] = t;
        }
    }
}

// sum of the per-brick partials in two fixed-order stages (deterministic): segment sums over
// blockIdx.y, then the sum of the segments
#define MN_SEG 64
__global__ void k_sum_parts(const float *__restrict__ part, int nblk, double *__restrict__ seg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MN_PPL) return;
    const int per = (nblk + MN_SEG - 1) / MN_SEG;
    const int b0 = blockIdx.y * per, b1 = min(nblk, b0 + per);
    double s = 0;
    for (int b = b0; b < b1; b++) s += part[(long)b * MN_PPL + i];
    seg[(long)blockIdx.y * MN_PPL + i] = s;
}
__global__ void k_sum_segs(const double *__restrict__ seg, float *__restrict__ grad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MN_PPL) return;
    double s = 0;
    for (int k = 0; k < MN_SEG; k++) s += seg[(long)k * MN_PPL + i];
    grad[i] = (float)s;
}

// network input: channels (delta / s0, phi1 / s1, phi2 / s2, 0, ...) from three FP32 grids
__global__ void k_pack_inputs(int N, int pitch, const float *__restrict__ a, const float *__restrict__ b,
                              const float *__restrict__ c, float ia, float ib, float ic, __nv_bfloat16 *__restrict__ out) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long nv = (long)N * N * N;
    if (v >= nv) return;
    const long row = v / N, z = v % N;
    const long src = row * pitch + z;
    __align__(16) __nv_bfloat16 vals[MN_C];
    vals[0] = __float2bfloat16_rn(a[src] * ia);
    vals[1] = __float2bfloat16_rn(b[src] * ib);
    vals[2] = __float2bfloat16_rn(c[src] * ic);
#pragma unroll
    for (int i = 3; i < MN_C; i++) vals[i] = __float2bfloat16_rn(0.f);
    uint4 *d = reinterpret_cast<uint4 *>(out + v * MN_C);
    d[0] = reinterpret_cast<const uint4 *>(vals)[0];
    d[1] = reinterpret_cast<const uint4 *>(vals)[1];
}

// MSE loss of pred (packed N^3, network units) against target / s_out (FP32 grid with pitch);
// writes dL/dpred into channel 0 of a BF16 tensor and adds the sum of squares to *loss
__global__ void k_mse(int N, int pitch, const float *__restrict__ pred, const float *__restrict__ target, float inv_s,
                      __nv_bfloat16 *__restrict__ dout, double *__restrict__ loss) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long nv = (long)N * N * N;
    double sq = 0;
    if (v < nv) {
        const long row = v / N, z = v % N;
        const float d = pred[v] - target[row * pitch + z] * inv_s;
        sq = (double)d * d;
        __align__(16) __nv_bfloat16 vals[MN_C];
        vals[0] = __float2bfloat16_rn(2.f * d / (float)nv);
#pragma unroll
        for (int i = 1; i < MN_C; i++) vals[i] = __float2bfloat16_rn(0.f);
        uint4 *o = reinterpret_cast<uint4 *>(dout + v * MN_C);
        o[0] = reinterpret_cast<const uint4 *>(vals)[0];
        o[1] = reinterpret_cast<const uint4 *>(vals)[1];
    }
    __shared__ double ws[32];
    for (int off = 16; off > 0; off >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, off);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = sq;
    __syncthreads();
    if (threadIdx.x < 32) {
        sq = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        for (int off = 16; off > 0; off >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, off);
        if (threadIdx.x == 0) atomicAdd(loss, sq);
    }
}

// BF16 operand layouts of all four layers from the FP32 parameters:
//   wf[l][t][co][ci] = W[l][t][ci][co]         (forward B operands)
//   wb[l][t][ci][co] = W[l][26 - t][ci][co]    (backward-data B operands: mirrored taps)
__global__ void k_prep_weights(const float *__restrict__ p, __nv_bfloat16 *__restrict__ wf, __nv_bfloat16 *__restrict__ wb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 4 * MN_WPL) return;
    const int l = i / MN_WPL, r = i % MN_WPL;
    const int t = r / (MN_C * MN_C), a = (r / MN_C) % MN_C, bq = r % MN_C;
    // r = (t*16 + a)*16 + bq, read as W[t][ci=a][co=bq]
    const float w = p[l * MN_PPL + r];
    wf[l * MN_WPL + (t * MN_C + bq) * MN_C + a] = __float2bfloat16_rn(w);
    wb[l * MN_WPL + ((26 - t) * MN_C + a) * MN_C + bq] = __float2bfloat16_rn(w);
}

// Adam (Kingma & Ba 2015) on the FP32 parameters; entries of padded channels stay zero
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m1, float *__restrict__ m2,
                       const unsigned char *__restrict__ live, float lr, float b1, float b2, float c1, float c2, float eps) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MANET_PARAMS || !live[i]) return;
    const float gi = g[i];
    const float m = b1 * m1[i] + (1.f - b1) * gi;
    const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = m;
    m2[i] = v;
    p[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

// ---- host side ----------------------------------------------------------------------------
static const int kCin[4] = {3, 16, 16, 16};
static const int kCout[4] = {16, 16, 16, 1};

struct ManetState {
    float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;
    unsigned char *live = nullptr;
    __nv_bfloat16 *wf = nullptr, *wb = nullptr;
    bool prepped = false;
    int warm_N = 0;  // grid of the warm-start inference (0: the solve's own grid)
};

static ManetState *state(const struct manet *net) { return reinterpret_cast<ManetState *>(net->priv); }

static bool live_param(int i) {
    const int l = i / MN_PPL, r = i % MN_PPL;
    if (r >= MN_WPL) return (r - MN_WPL) < kCout[l];
    const int ci = (r / MN_C) % MN_C, co = r % MN_C;
    return ci < kCin[l] && co < kCout[l];
}

static size_t conv_smem() { return (size_t)MN_TILE_VOX * 32 + 27 * MN_C * 32; }
static size_t wgrad_smem() { return (size_t)MN_TILE_VOX * 32 + (size_t)MN_BRICK_VOX * 32; }

static int check_n(int N) {
    if (N % MN_BZ || N % MN_BY || N % MN_BX || N < MN_BZ) {
        set_error(1, "network grids need N a multiple of %d (got %d)", MN_BZ, N);
        return 1;
    }
    return 0;
}

static int prep(ManetState *s) {
    if (s->prepped) return 0;
    k_prep_weights<<<(4 * MN_WPL + 255) / 256, 256, 0, stream()>>>(s->p, s->wf, s->wb);
    count_launch();
    MITOS_LAUNCH_CHECK("network weight layouts");
    s->prepped = true;
    return 0;
}

template <int MODE>
static int conv(int N, const __nv_bfloat16 *in, const __nv_bfloat16 *w, const float *bias, const __nv_bfloat16 *mask,
                __nv_bfloat16 *out, float *outf, int pitch, float scale) {
    static bool attr = false;
    const size_t smem = conv_smem();
    if (!attr) {
        MITOS_CUDA(cudaFuncSetAttribute(k_conv<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    const unsigned blocks = (unsigned)((N / MN_BX) * (N / MN_BY) * (N / MN_BZ));
    launch_begin(MODE == CONV_RELU ? "conv_relu" : MODE == CONV_LINEAR_OUT ? "conv_out" : "conv_bwd");
    k_conv<MODE><<<blocks, MN_THREADS, smem, stream()>>>(N, in, w, bias, mask, out, outf, pitch, scale);
    count_launch();
    MITOS_LAUNCH_CHECK("network convolution");
    return 0;
}

static int wgrad(int N, const __nv_bfloat16 *in, const __nv_bfloat16 *dout, float *part, float *grad) {
    static bool attr = false;
    const size_t smem = wgrad_smem();
    if (!attr) {
        MITOS_CUDA(cudaFuncSetAttribute(k_conv_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    const int blocks = (N / MN_BX) * (N / MN_BY) * (N / MN_BZ);
    launch_begin("conv_wgrad");
    k_conv_wgrad<<<blocks, MN_THREADS, smem, stream()>>>(N, in, dout, part);
    count_launch();
    MITOS_LAUNCH_CHECK("network weight gradient");
    double *seg = (double *)workspace(sizeof(double) * MN_SEG * MN_PPL, 129);
    if (!seg) return 5;
    launch_begin("wgrad_sum");
    k_sum_parts<<<dim3((MN_PPL + 127) / 128, MN_SEG), 128, 0, stream()>>>(part, blocks, seg);
    count_launch();
    k_sum_segs<<<(MN_PPL + 127) / 128, 128, 0, stream()>>>(seg, grad);
    count_launch();
    MITOS_LAUNCH_CHECK("network weight gradient sum");
    return 0;
}

// activations of one forward pass: act[0] input, act[1..3] hidden (BF16), pred (FP32 packed)
struct Acts {
    __nv_bfloat16 *act[4];
    float *pred;
};

static int acts(int N, Acts &A) {
    const size_t nv = (size_t)N * N * N;
    for (int l = 0; l < 4; l++) {
        A.act[l] = (__nv_bfloat16 *)workspace(nv * MN_C * sizeof(__nv_bfloat16), 120 + l);
        if (!A.act[l]) return 5;
    }
    A.pred = (float *)workspace(nv * sizeof(float), 124);
    return A.pred ? 0 : 5;
}

static int forward(ManetState *s, int N, Acts &A, float *outf, int pitch, float scale) {
    int e = prep(s);
    for (int l = 0; l < 3 && !e; l++)
        e = conv<CONV_RELU>(N, A.act[l], s->wf + l * MN_WPL, s->p + l * MN_PPL + MN_WPL, nullptr, A.act[l + 1], nullptr, 0, 1.f);
    if (!e)
        e = conv<CONV_LINEAR_OUT>(N, A.act[3], s->wf + 3 * MN_WPL, s->p + 3 * MN_PPL + MN_WPL, nullptr, nullptr,
                                  outf ? outf : A.pred, outf ? pitch : N, outf ? scale : 1.f);
    return e;
}

static int pack(const struct manet *net, int N, int pitch, const float *d, const float *p1, const float *p2, Acts &A) {
    const long nv = (long)N * N * N;
    launch_begin("net_pack");
    k_pack_inputs<<<(unsigned)((nv + 255) / 256), 256, 0, stream()>>>(N, pitch, d, p1, p2, 1.f / net->scale_in[0],
                                                                      1.f / net->scale_in[1], 1.f / net->scale_in[2], A.act[0]);
    count_launch();
    MITOS_LAUNCH_CHECK("network input");
    return 0;
}

// loss and gradients (s->g) of one sample; returns the mean squared error in *loss
static int loss_grad(const struct manet *net, int N, int pitch, const float *d, const float *p1, const float *p2,
                     const float *target, double *loss) {
    ManetState *s = state(net);
    Acts A;
    int e = acts(N, A);
    if (e) return e;
    const size_t nv = (size_t)N * N * N;
    __nv_bfloat16 *g0 = (__nv_bfloat16 *)workspace(nv * MN_C * sizeof(__nv_bfloat16), 125);
    __nv_bfloat16 *g1 = (__nv_bfloat16 *)workspace(nv * MN_C * sizeof(__nv_bfloat16), 126);
    const int blocks = (N / MN_BX) * (N / MN_BY) * (N / MN_BZ);
    float *part = (float *)workspace((size_t)blocks * MN_PPL * sizeof(float), 127);
    double *dl = (double *)workspace(sizeof(double), 128);
    if (!g0 || !g1 || !part || !dl) return 5;
    e = pack(net, N, pitch, d, p1, p2, A);
    if (!e) e = forward(s, N, A, nullptr, 0, 1.f);
    if (e) return e;
    MITOS_CUDA(cudaMemsetAsync(dl, 0, sizeof(double), stream()));
    launch_begin("net_mse");
    k_mse<<<(unsigned)((nv + 255) / 256), 256, 0, stream()>>>(N, pitch, A.pred, target, 1.f / net->scale_out, g0, dl);
    count_launch();
    MITOS_LAUNCH_CHECK("network loss");
    // backward: g0 = dL/d(output of layer l)
    for (int l = 3; l >= 0; l--) {
        e = wgrad(N, A.act[l], g0, part, s->g + l * MN_PPL);
        if (e) return e;
        if (l == 0) break;
        e = conv<CONV_BWD_MASK>(N, g0, s->wb + l * MN_WPL, nullptr, A.act[l], g1, nullptr, 0, 1.f);
        if (e) return e;
        std::swap(g0, g1);
    }
    MITOS_CUDA(cudaMemcpyAsync(loss, dl, sizeof(double), cudaMemcpyDeviceToHost, stream()));
    MITOS_CUDA(cudaStreamSynchronize(stream()));
    *loss /= (double)nv;
    return 0;
}

}  // namespace mitos

using namespace mitos;

extern "C" int manet_init(struct manet *net, unsigned long long seed) {
    if (!net) return 1;
    ManetState *s = new ManetState();
    const size_t pb = sizeof(float) * MANET_PARAMS;
    if (cudaMalloc(&s->p, pb) != cudaSuccess || cudaMalloc(&s->g, pb) != cudaSuccess ||
        cudaMalloc(&s->m1, pb) != cudaSuccess || cudaMalloc(&s->m2, pb) != cudaSuccess ||
        cudaMalloc(&s->live, MANET_PARAMS) != cudaSuccess ||
        cudaMalloc(&s->wf, sizeof(__nv_bfloat16) * 4 * MN_WPL) != cudaSuccess ||
        cudaMalloc(&s->wb, sizeof(__nv_bfloat16) * 4 * MN_WPL) != cudaSuccess) {
        cudaGetLastError();
        set_error(5, "out of device memory for the network");
        return 5;
    }
    // He-normal weights (std sqrt(2 / fan_in)), zero biases, from a splitmix64 stream
    std::vector<float> h(MANET_PARAMS, 0.f);
    std::vector<unsigned char> live(MANET_PARAMS, 0);
    uint64_t st = seed;
    auto next = [&st]() {
        uint64_t z = (st += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    };
    for (int i = 0; i < MANET_PARAMS; i++) {
        live[i] = live_param(i);
        const int l = i / MN_PPL, r = i % MN_PPL;
        if (!live[i] || r >= MN_WPL) continue;
        const double u1 = ((next() >> 11) + 0.5) * 0x1.0p-53, u2 = ((next() >> 11) + 0.5) * 0x1.0p-53;
        const double gss = sqrt(-2 * log(u1)) * cos(2 * M_PI * u2);
        h[i] = (float)(gss * sqrt(2.0 / (27.0 * kCin[l])));
    }
    MITOS_CUDA(cudaMemcpy(s->p, h.data(), pb, cudaMemcpyHostToDevice));
    MITOS_CUDA(cudaMemcpy(s->live, live.data(), MANET_PARAMS, cudaMemcpyHostToDevice));
    MITOS_CUDA(cudaMemset(s->m1, 0, pb));
    MITOS_CUDA(cudaMemset(s->m2, 0, pb));
    MITOS_CUDA(cudaMemset(s->g, 0, pb));
    net->priv = s;
    for (int c = 0; c < 3; c++) net->scale_in[c] = 1.f;
    net->scale_out = 1.f;
    net->steps = 0;
    return 0;
}

extern "C" int manet_free(struct manet *net) {
    if (!net || !net->priv) return 0;
    ManetState *s = state(net);
    cudaFree(s->p); cudaFree(s->g); cudaFree(s->m1); cudaFree(s->m2);
    cudaFree(s->live); cudaFree(s->wf); cudaFree(s->wb);
    delete s;
    net->priv = nullptr;
    return 0;
}

extern "C" int manet_get_params(const struct manet *net, float *host) {
    if (!net || !net->priv || !host) return 1;
    MITOS_CUDA(cudaMemcpy(host, state(net)->p, sizeof(float) * MANET_PARAMS, cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int manet_set_params(struct manet *net, const float *host) {
    if (!net || !net->priv || !host) return 1;
    ManetState *s = state(net);
    std::vector<float> h(host, host + MANET_PARAMS);
    for (int i = 0; i < MANET_PARAMS; i++)
        if (!live_param(i)) h[i] = 0.f;
    MITOS_CUDA(cudaMemcpy(s->p, h.data(), sizeof(float) * MANET_PARAMS, cudaMemcpyHostToDevice));
    s->prepped = false;
    return 0;
}

extern "C" int manet_get_grads(const struct manet *net, float *host) {
    if (!net || !net->priv || !host) return 1;
    MITOS_CUDA(cudaMemcpy(host, state(net)->g, sizeof(float) * MANET_PARAMS, cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int manet_loss_grad(struct manet *net, int N, int pitch, const float *delta, const float *phi1,
                               const float *phi2, const float *target, double *loss) {
    if (!net || !net->priv || !loss) return 1;
    if (check_n(N)) return 1;
    return loss_grad(net, N, pitch, delta, phi1, phi2, target, loss);
}

extern "C" int manet_train_step(struct manet *net, int N, int pitch, const float *delta, const float *phi1,
                                const float *phi2, const float *target, float lr, double *loss) {
    if (!net || !net->priv || !loss) return 1;
    if (check_n(N)) return 1;
    int e = loss_grad(net, N, pitch, delta, phi1, phi2, target, loss);
    if (e) return e;
    ManetState *s = state(net);
    net->steps++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)net->steps), c2 = 1.f - powf(b2, (float)net->steps);
    launch_begin("net_adam");
    k_adam<<<(MANET_PARAMS + 255) / 256, 256, 0, stream()>>>(s->p, s->g, s->m1, s->m2, s->live, lr, b1, b2, c1, c2, 1e-8f);
    count_launch();
    MITOS_LAUNCH_CHECK("network update");
    s->prepped = false;
    return 0;
}

extern "C" int manet_infer(struct manet *net, int N, int pitch, const float *delta, const float *phi1,
                           const float *phi2, float *out) {
    if (!net || !net->priv || !out) return 1;
    if (check_n(N)) return 1;
    Acts A;
    int e = acts(N, A);
    if (!e) e = pack(net, N, pitch, delta, phi1, phi2, A);
    if (!e) e = forward(state(net), N, A, out, pitch, net->scale_out);
    return e;
}

extern "C" int manet_set_warm_grid(struct manet *net, int Nw) {
    if (!net || !net->priv || Nw < 0 || (Nw && check_n(Nw))) {
        mitos::set_error(1, "manet_set_warm_grid: a grid size that is a multiple of 32 (or 0)");
        return 1;
    }
    state(net)->warm_N = Nw;
    return 0;
}

namespace mitos {
int manet_warm_grid(const struct manet *net) { return net && net->priv ? state(net)->warm_N : 0; }
}  // namespace mitos
