// fft_cluster.cu -- the Z and Y passes of a 3D r2c in one kernel (FP32, N = 256 and 512).
//
// A thread-block cluster of C CTAs owns one x-plane of the grid at a time (persistent: cluster c
// takes planes c, c + #clusters, ...).  Z step: CTA r transforms rows y in [r N/C, (r+1) N/C) of the
// real plane (an N/2-point complex FFT and the Hermitian split, as the Z r2c pass does) and stores
// each half-complex value straight into the shared memory of the CTA that owns its kz column
// (distributed shared memory: the x-plane's N x (N/2 + 1) values live across the cluster and never
// touch HBM).  After a cluster barrier, Y step: each CTA runs the length-N forward FFTs of its own
// kz columns and writes the plane's result rows.  The grid moves through HBM once in each
// direction: 2 G of traffic for the r2c's Z and Y steps instead of 4 G over two passes.
//
// The kz = 0 and kz = N/2 columns are real after the Z step; they travel as one complex column
// (kz = 0 in the real part, N/2 in the imaginary part), and their two transforms are separated
// after the Y FFT: F = FFT(a + i b), FFT(a)[k] = (F[k] + conj F[-k]) / 2, FFT(b)[k] =
// (F[k] - conj F[-k]) / 2i.  So each CTA owns exactly (N/2)/C columns.
//
// Column buffers: with two (NBUF = 2), alternating by plane, the Z step of plane i+1 writes the
// buffer the Y step of plane i-1 read, which every CTA finished before it passed plane i's cluster
// barrier: one barrier a plane.  With one, a second barrier after the Y step frees the buffer.
#include <cooperative_groups.h>

#include "fft_kernels.cuh"

namespace cg = cooperative_groups;

namespace mitos {

template <int NL, int C, int THREADS, int NBUF>
struct ZYShape {
    static constexpr int H2 = NL / 2;          // complex length of a row's FFT
    static constexpr int TPZ = H2 / 8;         // threads a row (E = 8)
    static constexpr int RZ = THREADS / TPZ;   // rows a Z step of the CTA
    static constexpr int RPC = NL / C;         // rows of a CTA
    static constexpr int ZIT = RPC / RZ;       // Z steps a plane
    static constexpr int ZB = ZIT < 2 ? ZIT : 2;  // Z steps whose rows are loaded together
    static constexpr int CPC = H2 / C;         // kz columns of a CTA
    static constexpr int P = THREADS * 8 / NL; // pencils a Y round
    static constexpr int YR = CPC / P;         // Y rounds
    // column pitch CP = 16/P mod 16: a half-warp's 16 lanes (P pencils x 16/P consecutive y) read
    // 16 distinct 8-byte bank pairs
    static constexpr int CP = NL + 16 / P;
    static constexpr int ZS = H2 + H2 / 8 + 1;  // spad_len(H2)
    static constexpr int YS = NL + NL / 8 + 1;  // spad_len(NL)
    static constexpr int SCR = (RZ * ZS > P * YS) ? RZ * ZS : P * YS;
    static constexpr size_t smem() { return sizeof(float2) * ((size_t)NBUF * CPC * CP + SCR + NL); }
    static_assert(P * (NL / 8) == THREADS && P <= 16, "a Y round is one pencil group of the whole block");
    static_assert(ZIT * RZ == RPC && ZIT % ZB == 0 && YR * P == CPC && CPC * C == H2, "shape");
};

template <int NL, int C, int THREADS, int NBUF>
__global__ void __launch_bounds__(THREADS, THREADS == 256 ? 2 : 1) k_zy_r2c_cluster(GridGeom g, PassArgs a) {
    using S = ZYShape<NL, C, THREADS, NBUF>;
    using T = float;
    constexpr int P = S::P;
    extern __shared__ __align__(16) unsigned char smraw[];
    cplx<T> *colbuf = reinterpret_cast<cplx<T> *>(smraw);  // [NBUF][CPC][CP]
    cplx<T> *scr = colbuf + NBUF * S::CPC * S::CP;         // FFT exchange (Z rows, then Y pencils)
    cplx<T> *pk = scr + S::SCR;                            // the packed kz = 0 | N/2 column's FFT
    cg::cluster_group cl = cg::this_cluster();
    const int r = (int)cl.block_rank();
    const int cid = blockIdx.x / C, ncl = gridDim.x / C;
    const int tid = threadIdx.x;
    const size_t bo = (size_t)blockIdx.y * (size_t)a.bstride;
    const T *in = bat<const T>(a.in[0], bo);
    cplx<T> *out = bat<cplx<T>>(a.out[0], bo);
    const cplx<T> *tw = reinterpret_cast<const cplx<T> *>(g.twN);
    const T ra = a.frho_a, rb = a.frho_b, scale = a.fscale;
    const bool affine = ra != (T)1 || rb != (T)0;
    constexpr int H = NL / 2 + 1;
    // Z step lanes: row pr of the step, thread tz of the row
    const int pr = tid / S::TPZ, tz = tid % S::TPZ;
    cplx<T> *zs = scr + pr * S::ZS;
    // Y step lanes: pencil p (fastest), thread ty of the pencil
    const int p = tid % P, ty = tid / P;
    cl.sync();  // every CTA of the cluster runs before the first remote store
    int buf = 0;
#pragma unroll 1
    for (int x = cid; x < NL; x += ncl, buf = (NBUF == 2) ? buf ^ 1 : 0) {
        cplx<T> *cb = colbuf + buf * S::CPC * S::CP;
        // ---- Z: rows -> half-complex values into the owners' column buffers ----
#pragma unroll 1
        for (int z0 = 0; z0 < S::ZIT; z0 += S::ZB) {
            cplx<T> v[S::ZB][8];
#pragma unroll
            for (int zi = 0; zi < S::ZB; zi++) {
                const int y = r * S::RPC + (z0 + zi) * S::RZ + pr;
                const T *src = in + ((long)x * NL + y) * a.rp_in;
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    cplx<T> z = *reinterpret_cast<const cplx<T> *>(src + 2 * n_in_ct<S::H2, 8>(tz, e));
                    if (affine) z = mk<T>(z.x * ra + rb, z.y * ra + rb);
                    v[zi][e] = z;
                }
            }
#pragma unroll
            for (int zi = 0; zi < S::ZB; zi++) {
                const int y = r * S::RPC + (z0 + zi) * S::RZ + pr;
                fft_regs_ct<T, 8, -1, S::H2, 1>(v[zi], zs, tz, reinterpret_cast<const cplx<T> *>(g.plH.twst));
#pragma unroll
                for (int e = 0; e < 8; e++) zs[xpos<S::H2, 1>(n_out_ct<S::H2, 8>(tz, e))] = v[zi][e];
                pencil_sync<S::H2, 8, 1>();
                T dc = 0;
                for (int k = tz; k <= S::H2; k += S::TPZ) {
                    const cplx<T> Z = zs[xpos<S::H2, 1>(k == S::H2 ? 0 : k)];
                    const cplx<T> Zc = zs[xpos<S::H2, 1>(k == 0 ? 0 : S::H2 - k)];
                    const cplx<T> ev = mk<T>((T)0.5 * (Z.x + Zc.x), (T)0.5 * (Z.y - Zc.y));
                    const cplx<T> od = mk<T>((T)0.5 * (Z.y + Zc.y), (T)-0.5 * (Z.x - Zc.x));
                    const cplx<T> X = cadd<T>(ev, cmul<T>(od, __ldg(tw + k)));
                    if (k == 0) {
                        dc = X.x;  // thread 0 of the row also takes k = N/2, its last value
                    } else if (k == S::H2) {
                        *cl.map_shared_rank(cb + y, 0) = mk<T>(dc, X.x);
                    } else {
                        const int owner = k / S::CPC, j = k % S::CPC;
                        *cl.map_shared_rank(cb + j * S::CP + y, owner) = X;
                    }
                }
                pencil_sync<S::H2, 8, 1>();  // the row's exchange slots are free for the next row
            }
        }
        cl.sync();  // the plane's columns are complete in every CTA
        // ---- Y: forward FFTs of this CTA's columns, rows of the plane out ----
#pragma unroll 1
        for (int yr = 0; yr < S::YR; yr++) {
            const int j = yr * P + p;
            const int kz = r * S::CPC + j;
            const cplx<T> *col = cb + j * S::CP;
            cplx<T> w[8];
#pragma unroll
            for (int e = 0; e < 8; e++) w[e] = col[n_in_ct<NL, 8>(ty, e)];
            fft_regs_ct<T, 8, -1, NL, P>(w, scr + p, ty, reinterpret_cast<const cplx<T> *>(g.plN.twst));
            const bool packed = r == 0 && j == 0;
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const int ky = n_out_ct<NL, 8>(ty, e);
                if (packed) pk[ky] = w[e];
                else out[((long)x * NL + ky) * H + kz] = cscale<T>(w[e], scale);
            }
            if (r == 0 && yr == 0) {  // uniform in the CTA
                __syncthreads();
                for (int i = tid; i < NL; i += THREADS) {
                    const cplx<T> F = pk[i], Fc = pk[i == 0 ? 0 : NL - i];
                    const cplx<T> A = mk<T>((T)0.5 * (F.x + Fc.x), (T)0.5 * (F.y - Fc.y));
                    const cplx<T> B = mk<T>((T)0.5 * (F.y + Fc.y), (T)-0.5 * (F.x - Fc.x));
                    cplx<T> *row = out + ((long)x * NL + i) * H;
                    row[0] = cscale<T>(A, scale);
                    row[S::H2] = cscale<T>(B, scale);
                }
            }
        }
        if constexpr (NBUF == 1) cl.sync();  // every CTA has read its columns: the buffer is free
    }
}

template <int NL, int C, int THREADS, int NBUF>
static int launch_zy(const GridGeom &g, const PassArgs &a) {
    using S = ZYShape<NL, C, THREADS, NBUF>;
    auto kern = k_zy_r2c_cluster<NL, C, THREADS, NBUF>;
    static int max_clusters = -1;  // per instantiation, for the current device
    const size_t smem = S::smem();
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream();
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (max_clusters < 0) {
        MITOS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        if (C > 8) MITOS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        cfg.gridDim = dim3(C * 64);
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
            cudaGetLastError();
            n = 0;
        }
        max_clusters = n;
    }
    if (max_clusters < 1) return -1;  // no cluster of this shape fits: the two-pass route
    const int nb = a.batch > 1 ? a.batch : 1;
    int ncl = max_clusters / nb;
    if (ncl < 1) ncl = 1;
    if (ncl > NL) ncl = NL;
    cfg.gridDim = dim3((unsigned)(ncl * C), (unsigned)nb);
    launch_begin("zy_r2c");
    const PassArgs af = with_f32(a);
    MITOS_CUDA(cudaLaunchKernelEx(&cfg, kern, g, af));
    count_launch();
    MITOS_LAUNCH_CHECK("cluster Z + Y r2c pass");
    return 0;
}

// 0: off; 1..3: the cluster shapes below (1: C = 16 CTAs of 512 threads, two column buffers;
// 2: C = 16 of 256 threads, one buffer, two CTAs an SM; 3: C = 8 of 512 threads, one buffer)
static int g_cluster_fft = 0;
void set_cluster_fft(int mode) { g_cluster_fft = mode; }
int cluster_fft() { return g_cluster_fft; }

// the r2c's Z and Y steps in one cluster pass where the shape has one; -1 where it has none (the
// caller runs the Z r2c and Y passes)
int launch_zy_r2c(const GridGeom &g, int precision, const PassArgs &a) {
    const int m = g_cluster_fft;
    if (!m || precision != MITOS_FP32 || g.E != 8 || g.custom_radix) return -1;
    if ((a.rp_in & 1) || ((uintptr_t)a.in[0] & 7)) return -1;
    if (g.N == 512) {
        if (m == 1) return launch_zy<512, 16, 512, 2>(g, a);
        if (m == 2) return launch_zy<512, 16, 256, 1>(g, a);
        if (m == 3) return launch_zy<512, 8, 512, 1>(g, a);
    }
    if (g.N == 256) {
        if (m == 1) return launch_zy<256, 8, 512, 2>(g, a);
        if (m == 2) return launch_zy<256, 8, 256, 1>(g, a);
        if (m == 3) return launch_zy<256, 4, 512, 1>(g, a);
    }
    return -1;
}

}  // namespace mitos
