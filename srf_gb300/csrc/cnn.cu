// BF16 3-D convolution network kernels with FP32 accumulation (scatter surrogate; not in the
// reference).
//
// Activations are NDHWC bfloat16 with an explicit channel stride and offset, so a layer can
// read or write a channel slice of a wider buffer (U-Net skip concatenation costs nothing).
// Weights are [Cout][27][Cin] bfloat16 (tap-major within an output channel), FP32 master copies
// live in the optimiser.
//
// conv3d 3x3x3 (pad 1, stride 1) is an implicit GEMM: rows = output voxels, columns = output
// channels, K = 27 taps x Cin, walked in (tap, 16-channel chunk) steps. For each step the
// gathered input rows (zero outside the volume) and the weight slice are staged in shared memory
// and the warps issue mma.sync.m16n8k16 BF16 tensor-core products into FP32 accumulators. The
// tile follows the layer: 64 voxels x 64 channels or 128 x 32 when the grid fills the GPU
// (double-buffered, one barrier per step), else 64 x 32 with the K steps dealt round-robin to the
// CTA's 4 warps and their partial tiles summed at the end. The data gradient is the same kernel
// on flipped, transposed weights. The weight gradient is a split-K GEMM over voxels per tap,
// accumulated with FP32 atomics. Requirements (checked on the host): Cin and Cout multiples of
// 16, channel strides and offsets multiples of 8 (16-byte aligned rows).
#include <algorithm>
#include <cstring>
#include <cuda.h>
#include <cuda_bf16.h>

#include "common.cuh"

namespace srf {

constexpr int kCM = 64, kCN = 64, kCK = 16, kCPad = 24;  // tile sizes, padded smem row (bf16)

struct Act {  // NDHWC view
    int n, d, h, w, cstride, coff;
};

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t lds32(const __nv_bfloat16 *p) {
    return *reinterpret_cast<const uint32_t *>(p);
}

// One k-step of a warp: A rows [r0, r0+16) of As, B columns [0, 64) of Bs (stored [n][k]).
__device__ __forceinline__ void warp_mma_step(const __nv_bfloat16 (*As)[kCPad],
                                              const __nv_bfloat16 (*Bs)[kCPad], int r0,
                                              float (&acc)[8][4]) {
    const int lane = threadIdx.x & 31, grp = lane >> 2, tig = lane & 3;
    uint32_t a[4];
    a[0] = lds32(&As[r0 + grp][tig * 2]);
    a[1] = lds32(&As[r0 + grp + 8][tig * 2]);
    a[2] = lds32(&As[r0 + grp][tig * 2 + 8]);
    a[3] = lds32(&As[r0 + grp + 8][tig * 2 + 8]);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        uint32_t b[2];
        b[0] = lds32(&Bs[j * 8 + grp][tig * 2]);
        b[1] = lds32(&Bs[j * 8 + grp][tig * 2 + 8]);
        mma_bf16(acc[j], a, b);
    }
}

// One k-step of a warp on a BM x BN tile: MT 16-row m-tiles from row r0 of As, NT 8-column
// n-tiles of Bs (stored [n][k]).
template <int MT, int NT>
__device__ __forceinline__ void warp_mma_tile(const __nv_bfloat16 (*As)[kCPad], const __nv_bfloat16 (*Bs)[kCPad],
                                              int r0, float (&acc)[MT][NT][4]) {
    const int lane = threadIdx.x & 31, grp = lane >> 2, tig = lane & 3;
    uint32_t a[MT][4];
#pragma unroll
    for (int m = 0; m < MT; ++m) {
        const int r = r0 + m * 16 + grp;
        a[m][0] = lds32(&As[r][tig * 2]);
        a[m][1] = lds32(&As[r + 8][tig * 2]);
        a[m][2] = lds32(&As[r][tig * 2 + 8]);
        a[m][3] = lds32(&As[r + 8][tig * 2 + 8]);
    }
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        uint32_t b[2];
        b[0] = lds32(&Bs[j * 8 + grp][tig * 2]);
        b[1] = lds32(&Bs[j * 8 + grp][tig * 2 + 8]);
#pragma unroll
        for (int m = 0; m < MT; ++m) mma_bf16(acc[m][j], a[m], b);
    }
}

// y[v, co] = act(b[co] + sum_{tap, ci} x[v + tap - 1, ci] w[co, tap, ci]) on BM-voxel x
// BN-channel tiles (4 warps, each BM/4 rows x BN columns). K runs over (tap, 16-channel chunk)
// steps; the next step's gathered rows and weight slice are loaded into registers while the
// tensor cores work on the current one and are stored into the other of two shared-memory
// buffers, so each step costs one barrier and no exposed global latency.
template <int BM, int BN>
__global__ void __launch_bounds__(128)
k_conv3d_fwd(const __nv_bfloat16 *__restrict__ x, Act xa, int cin, const __nv_bfloat16 *__restrict__ wt,
             const float *__restrict__ bias, int cout, int relu, __nv_bfloat16 *__restrict__ y, Act ya,
             float *__restrict__ yf) {
    constexpr int MT = BM / 64, NT = BN / 8;  // m-tiles per warp, n-tiles
    constexpr int AS = BM / 64;               // A slots (half rows of 8 channels) per thread
    static_assert(2 * BN <= 128, "one B slot per thread");
    __shared__ __align__(16) __nv_bfloat16 As[2][BM][kCPad];
    __shared__ __align__(16) __nv_bfloat16 Bs[2][BN][kCPad];
    const int64_t nvox = (int64_t)xa.d * xa.h * xa.w;
    const int64_t v0 = (int64_t)blockIdx.x * BM;
    const int co0 = blockIdx.y * BN;
    const int nb = blockIdx.z;
    const int tid = threadIdx.x, warp = tid >> 5;
    const __nv_bfloat16 *xb = x + (int64_t)nb * nvox * xa.cstride + xa.coff;
    // A slots: row tid / 2 + 64 i, channel half (tid & 1) * 8
    const int lh = (tid & 1) * 8;
    int lr[AS], lz[AS], ly[AS], lx[AS];
    bool lok[AS];
#pragma unroll
    for (int i = 0; i < AS; ++i) {
        lr[i] = (tid >> 1) + 64 * i;
        const int64_t v = v0 + lr[i];
        lok[i] = v < nvox;
        const int z = lok[i] ? (int)(v / ((int64_t)xa.h * xa.w)) : 0;
        const int rem = lok[i] ? (int)(v - (int64_t)z * xa.h * xa.w) : 0;
        lz[i] = z;
        ly[i] = rem / xa.w;
        lx[i] = rem - ly[i] * xa.w;
    }
    // B slot: threads [0, 2 BN) load output channel co0 + tid / 2
    const bool bload = tid < 2 * BN;
    const int br = tid >> 1, bco = co0 + br;
    const bool bok = bload && bco < cout;
    uint4 ra[AS], rb = make_uint4(0, 0, 0, 0);
    auto load = [&](int tap, int c0) {
        const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
#pragma unroll
        for (int i = 0; i < AS; ++i) {
            const int zz = lz[i] + dz, yy = ly[i] + dy, xx = lx[i] + dx;
            const bool in = lok[i] && zz >= 0 && zz < xa.d && yy >= 0 && yy < xa.h && xx >= 0 && xx < xa.w;
            ra[i] = make_uint4(0, 0, 0, 0);
            if (in) ra[i] = *reinterpret_cast<const uint4 *>(xb + (((int64_t)zz * xa.h + yy) * xa.w + xx) * xa.cstride + c0 + lh);
        }
        rb = make_uint4(0, 0, 0, 0);
        if (bok) rb = *reinterpret_cast<const uint4 *>(wt + ((int64_t)bco * 27 + tap) * cin + c0 + lh);
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int i = 0; i < AS; ++i) *reinterpret_cast<uint4 *>(&As[buf][lr[i]][lh]) = ra[i];
        if (bload) *reinterpret_cast<uint4 *>(&Bs[buf][br][lh]) = rb;
    };
    float acc[MT][NT][4] = {};
    const int nck = cin / kCK, steps = 27 * nck;
    int tap = 0, ck = 0;
    load(0, 0);
    store(0);
    __syncthreads();
    for (int s = 0; s < steps; ++s) {
        const int cur = s & 1;
        int ntap = tap, nc = ck + 1;
        if (nc == nck) {
            nc = 0;
            ++ntap;
        }
        const bool more = s + 1 < steps;
        if (more) load(ntap, nc * kCK);
        warp_mma_tile<MT, NT>(As[cur], Bs[cur], warp * (BM / 4), acc);
        if (more) store(cur ^ 1);
        __syncthreads();
        tap = ntap;
        ck = nc;
    }
    // epilogue: rows warp * BM/4 + 16 m + grp (+8), columns co0 + 8 j + 2 tig (+1)
    const int lane = tid & 31, grp = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        const int co = co0 + j * 8 + tig * 2;
        if (co >= cout) continue;
        const float b0 = bias ? bias[co] : 0.0f, b1 = bias ? bias[co + 1] : 0.0f;
#pragma unroll
        for (int m = 0; m < MT; ++m)
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                const int64_t v = v0 + warp * (BM / 4) + m * 16 + grp + half * 8;
                if (v >= nvox) continue;
                float r0 = acc[m][j][half * 2] + b0, r1 = acc[m][j][half * 2 + 1] + b1;
                if (relu) {
                    r0 = fmaxf(r0, 0.0f);
                    r1 = fmaxf(r1, 0.0f);
                }
                const int64_t o = ((int64_t)nb * nvox + v) * ya.cstride + ya.coff + co;
                *reinterpret_cast<__nv_bfloat162 *>(y + o) = __floats2bfloat162_rn(r0, r1);
                if (yf) {
                    yf[o] = r0;
                    yf[o + 1] = r1;
                }
            }
    }
}

// ---------------------------------------------------------------- tcgen05 variant
// The 128-voxel x 32-channel tile on the 5th-generation tensor cores: each (tap, 16-channel) K
// step's gathered input rows (A, 128 x 16) and weight slice (B, 32 x 16) are written into one of
// kTcStages shared-memory stages in the canonical no-swizzle K-major layout (8-row x 16-byte core
// matrices; K-adjacent core matrices 128 B apart, 8-row groups 256 B apart); one thread issues
// tcgen05.mma (kind::f16, BF16 inputs, FP32 accumulator in tensor memory, M = 128, N = 32) and
// commits it to the stage's mbarrier, which the threads wait on before refilling that stage.
// The next step's global loads are in flight meanwhile. The accumulator (128 lanes x 32 columns
// of TMEM) is read back with tcgen05.ld for the bias/activation epilogue. Every wait is bounded:
// on a timeout the kernel records it in g_tc_status, waits (bounded) for its last commit, frees
// its tensor memory and returns.
constexpr int kTcStages = 4;
constexpr int kTcM = 128, kTcN = 32;
constexpr int kTcABytes = kTcM * kCK * 2, kTcBBytes = kTcN * kCK * 2;  // 4096, 1024
constexpr uint32_t kTcCols = 32;                                       // TMEM columns (FP32 N)
constexpr int kTcSpin = 1 << 20;                                       // mbarrier polls before giving up

__device__ int g_tc_status;  // 0, or 1 when a tcgen05 conv launch gave up waiting

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (int i = 0; i < kTcSpin; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}

// Shared-memory matrix descriptor (no swizzle, K-major): start address, leading (K-direction)
// and stride (8-row direction) byte offsets, all >> 4; bit 46 set (descriptor version).
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B (bits 7-9,
// 10-12 = 1), both K-major, N >> 3 in bits 17-22, M >> 4 in bits 24-28.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                              ((uint32_t)(kTcM >> 4) << 24);

__global__ void __launch_bounds__(128, 4)
k_conv3d_fwd_tc(const __nv_bfloat16 *__restrict__ x, Act xa, int cin, const __nv_bfloat16 *__restrict__ wt,
                const float *__restrict__ bias, int cout, int relu, __nv_bfloat16 *__restrict__ y, Act ya,
                float *__restrict__ yf) {
    __shared__ __align__(1024) unsigned char sA[kTcStages][kTcABytes];
    __shared__ __align__(1024) unsigned char sB[kTcStages][kTcBBytes];
    __shared__ __align__(8) uint64_t bars[kTcStages];
    __shared__ uint32_t tmem_slot;
    __shared__ int gave_up;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int64_t nvox = (int64_t)xa.d * xa.h * xa.w;
    const int64_t v0 = (int64_t)blockIdx.x * kTcM;
    const int co0 = blockIdx.y * kTcN;
    const int nb = blockIdx.z;
    const __nv_bfloat16 *xb = x + (int64_t)nb * nvox * xa.cstride + xa.coff;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&tmem_slot)), "r"(kTcCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid < kTcStages)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&bars[tid])) : "memory");
    if (tid == 0) gave_up = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    // A row of this thread: voxel v0 + tid; B row (threads 0-63): channel co0 + tid / 2, half tid & 1
    const int64_t v = v0 + tid;
    const bool vok = v < nvox;
    const int z = vok ? (int)(v / ((int64_t)xa.h * xa.w)) : 0;
    const int rem = vok ? (int)(v - (int64_t)z * xa.h * xa.w) : 0;
    const int yy0 = rem / xa.w, xx0 = rem - (rem / xa.w) * xa.w;
    const bool bload = tid < 2 * kTcN;
    const int bn = tid >> 1, bh = tid & 1;
    const bool bok = bload && co0 + bn < cout;
    // canonical offsets: row r -> (r / 8) * 256 + (r % 8) * 16, K-half h -> + h * 128
    const uint32_t aoff = (uint32_t)((tid >> 3) * 256 + (tid & 7) * 16);
    const uint32_t boff = (uint32_t)((bn >> 3) * 256 + (bn & 7) * 16 + bh * 128);

    uint4 ra0, ra1, rb;
    auto load = [&](int tap, int c0) {
        const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
        const int zz = z + dz, yy = yy0 + dy, xx = xx0 + dx;
        const bool in = vok && zz >= 0 && zz < xa.d && yy >= 0 && yy < xa.h && xx >= 0 && xx < xa.w;
        ra0 = ra1 = make_uint4(0, 0, 0, 0);
        if (in) {
            const __nv_bfloat16 *p = xb + (((int64_t)zz * xa.h + yy) * xa.w + xx) * xa.cstride + c0;
            ra0 = *reinterpret_cast<const uint4 *>(p);
            ra1 = *reinterpret_cast<const uint4 *>(p + 8);
        }
        rb = make_uint4(0, 0, 0, 0);
        if (bok) rb = *reinterpret_cast<const uint4 *>(wt + ((int64_t)(co0 + bn) * 27 + tap) * cin + c0 + 8 * bh);
    };

    const int nck = cin / kCK, steps = 27 * nck;
    int tap = 0, ck = 0;
    load(0, 0);
    for (int s = 0; s < steps; ++s) {
        const int st = s % kTcStages;
        if (s >= kTcStages) {  // the MMA that read this stage kTcStages steps ago has completed
            if (!mbar_wait(smem_u32(&bars[st]), (uint32_t)((s / kTcStages - 1) & 1))) {
                gave_up = 1;  // benign race: every writer stores 1
            }
        }
        __syncthreads();
        if (gave_up) break;
        *reinterpret_cast<uint4 *>(&sA[st][aoff]) = ra0;
        *reinterpret_cast<uint4 *>(&sA[st][aoff + 128]) = ra1;
        if (bload) *reinterpret_cast<uint4 *>(&sB[st][boff]) = rb;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        int ntap = tap, nc = ck + 1;
        if (nc == nck) {
            nc = 0;
            ++ntap;
        }
        if (s + 1 < steps) load(ntap, nc * kCK);
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint64_t ad = tc_desc(smem_u32(sA[st]), 128, 256);
            const uint64_t bd = tc_desc(smem_u32(sB[st]), 128, 256);
            const uint32_t acc = s > 0 ? 1u : 0u;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                :: "r"(tmem), "l"(ad), "l"(bd), "r"(kTcIdesc), "r"(acc) : "memory");
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(smem_u32(&bars[st])) : "memory");
        }
        tap = ntap;
        ck = nc;
    }
    // the last commit covers every MMA issued before it
    const int issued = gave_up ? 0 : steps;
    bool ok = !gave_up;
    if (issued > 0) {
        const int last = issued - 1;
        ok = mbar_wait(smem_u32(&bars[last % kTcStages]), (uint32_t)((last / kTcStages) & 1)) && ok;
    } else if (tid == 0) {
        // a timeout left MMAs in flight: wait (bounded) on every stage's pending phase
        for (int st = 0; st < kTcStages; ++st) mbar_wait(smem_u32(&bars[st]), 0);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (vok) {
            const int64_t o = ((int64_t)nb * nvox + v) * ya.cstride + ya.coff + co0;
#pragma unroll
            for (int j = 0; j < kTcN; j += 8) {
                if (co0 + j >= cout) break;
                float f[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    float t = __uint_as_float(r[j + e]) + (bias ? bias[co0 + j + e] : 0.0f);
                    f[e] = relu ? fmaxf(t, 0.0f) : t;
                }
                __nv_bfloat162 h[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) h[e] = __floats2bfloat162_rn(f[2 * e], f[2 * e + 1]);
                *reinterpret_cast<uint4 *>(y + o + j) = *reinterpret_cast<const uint4 *>(h);
                if (yf) {
#pragma unroll
                    for (int e = 0; e < 8; ++e) yf[o + j + e] = f[e];
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(&g_tc_status, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kTcCols) : "memory");
}

static int g_conv_tc = 1;    // srf_set_conv_tc: 0 mma.sync, 1 tcgen05 K-step tiles, 2/3 also halo tiles (cp.async / TMA)
static int g_conv_path = -1;  // kernel of the last srf_conv3d_fwd launch (srf_conv_last_path)

// ---------------------------------------------------------------- tcgen05 + TMA, halo tiles
// Batch-1 layers on wide grids (W >= 96, Cout = 32): an output tile is 128 consecutive voxels of
// one x-row. Its input halo (rows x0 - 1 .. x0 + 128 of the 3 x 3 (z, y) neighbour rows, 16
// channels per group) is one TMA box per 8-channel chunk, written by the TMA unit in the
// canonical no-swizzle K-major layout [chunk][z][y][x][8 channels] (rows 16 B apart, zero fill
// outside the volume = the convolution's padding; TMA = false: the same layout written by the
// threads with zero-filling cp.async). Every tap's A operand is then the same halo
// at a row offset: descriptor start = halo + ((dz + 1) * 3 + dy + 1) * 130 rows + dx + 1, so the
// 27 taps of a 16-channel group are 27 back-to-back tcgen05.mma with no gather and no barrier
// between them. The weights of the group (B, [chunk][tap][co][8]) are staged with cp.async by all
// threads. Persistent CTAs (one per SM) walk (tile, group) items through two stages: the next
// item's TMA and cp.async copies are in flight while the tensor cores work on the current one;
// a stage is refilled when the mbarrier its MMAs committed to has fired. The accumulator lives
// in 32 TMEM columns; after a tile's last group it is read with tcgen05.ld for the bias and
// activation epilogue. Bounded waits as in k_conv3d_fwd_tc. The TMA form measured slower than
// the K-step kernels on the surrogate's level-1 layers (62 against 33-43 us at Cin 16): a TMA
// box whose inner extent is one 16-byte channel chunk moves 2,340 separate rows per halo.
constexpr int kHx = 130;                               // halo rows along x
constexpr int kHPlane = 9 * kHx * 16;                  // one 8-channel chunk of the halo: 18,720 B
constexpr int kHPlanePad = (kHPlane + 127) / 128 * 128;  // TMA destinations are 128-byte aligned
constexpr int kHABytes = 2 * kHPlanePad;               // a 16-channel group
constexpr int kHBBytes = 2 * 27 * kTcN * 16;           // [chunk][tap][co][16 B] = 27,648 B
constexpr int kHStage = kHABytes + kHBBytes;
constexpr int kHMaxChunks = 16;                        // Cin <= 128
constexpr int kHSmem = 2 * kHStage + 1024;             // two stages + alignment slack

struct HaloMaps {
    CUtensorMap m[kHMaxChunks];  // chunk c: dims (8 channels, W, H, D) from channel 8c of the slice
};

template <bool TMA>
__global__ void __launch_bounds__(256, 1)
k_conv3d_fwd_halo(const __grid_constant__ HaloMaps maps, const __nv_bfloat16 *__restrict__ x, Act xa, int cin,
                  const __nv_bfloat16 *__restrict__ wt, const float *__restrict__ bias, int relu,
                  __nv_bfloat16 *__restrict__ y, Act ya, float *__restrict__ yf) {
    extern __shared__ unsigned char dsm[];
    __shared__ __align__(8) uint64_t full[2], empty[2], done;
    __shared__ uint32_t tmem_slot;
    __shared__ int gave_up;
    unsigned char *base = (unsigned char *)(((uintptr_t)dsm + 1023) & ~(uintptr_t)1023);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int G = cin / 16;
    const int tx = (xa.w + kTcM - 1) / kTcM;
    const int64_t n_tiles = (int64_t)xa.d * xa.h * tx;
    const int64_t my_tiles = n_tiles > blockIdx.x ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int64_t items = my_tiles * G;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&tmem_slot)), "r"(kTcCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid < 2) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&full[tid])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&empty[tid])) : "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&done)) : "memory");
        gave_up = 0;
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    auto tile_of = [&](int64_t it, int &z, int &yy, int &x0) {
        const int64_t t = blockIdx.x + (it / G) * (int64_t)gridDim.x;
        const int xt = (int)(t % tx);
        const int64_t zy = t / tx;
        yy = (int)(zy % xa.h);
        z = (int)(zy / xa.h);
        x0 = xt * kTcM;
    };
    // copies of item `it` into stage st: TMA of the two halo chunks (thread 0), weights (all)
    auto issue = [&](int64_t it, int st) {
        int z, yy, x0;
        tile_of(it, z, yy, x0);
        const int g = (int)(it % G);
        unsigned char *sa = base + st * kHStage, *sb = sa + kHABytes;
        const uint32_t fb = smem_u32(&full[st]);
        if (TMA && tid == 0) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                         :: "r"(fb), "r"((uint32_t)(2 * kHPlane)) : "memory");
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const uint64_t map = reinterpret_cast<uint64_t>(&maps.m[2 * g + c]);
                asm volatile(
                    "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                    " [%0], [%1, {%2, %3, %4, %5}], [%6];"
                    :: "r"(smem_u32(sa + c * kHPlanePad)), "l"(map), "r"(0), "r"(x0 - 1), "r"(yy - 1), "r"(z - 1),
                       "r"(fb) : "memory");
            }
        }
        if (!TMA) {  // the halo rows by the threads, zero outside the volume
            const __nv_bfloat16 *xg = x + xa.coff + 16 * g;
            for (int j = tid; j < 2 * 9 * kHx; j += blockDim.x) {  // j = chunk * 1170 + row
                const int c = j / (9 * kHx), r = j - c * (9 * kHx);
                const int gz = z - 1 + r / (3 * kHx), gy = yy - 1 + (r / kHx) % 3, gx = x0 - 1 + r % kHx;
                const bool in = gz >= 0 && gz < xa.d && gy >= 0 && gy < xa.h && gx >= 0 && gx < xa.w;
                const __nv_bfloat16 *src = in ? xg + (((int64_t)gz * xa.h + gy) * xa.w + gx) * xa.cstride + 8 * c : x;
                asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;"
                             :: "r"(smem_u32(sa + c * kHPlanePad + r * 16)), "l"(src), "r"(in ? 16u : 0u) : "memory");
            }
        }
        for (int j = tid; j < 2 * 27 * kTcN; j += blockDim.x) {  // j = (chunk * 27 + tap) * 32 + co
            const int co = j & (kTcN - 1), tap = (j >> 5) % 27, c = (j >> 5) / 27;
            const __nv_bfloat16 *src = wt + ((int64_t)co * 27 + tap) * cin + 16 * g + 8 * c;
            asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" :: "r"(smem_u32(sb + j * 16)), "l"(src) : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };

    if (items > 0) issue(0, 0);
    int tiles_done = 0;
    for (int64_t it = 0; it < items; ++it) {
        const int st = (int)(it & 1);
        const int g = (int)(it % G);
        if (it + 1 < items) {
            if (it >= 1 && !mbar_wait(smem_u32(&empty[st ^ 1]), (uint32_t)(((it - 1) >> 1) & 1))) gave_up = 1;
            else issue(it + 1, st ^ 1);
        } else {
            asm volatile("cp.async.commit_group;" ::: "memory");
        }
        asm volatile("cp.async.wait_group 1;" ::: "memory");  // item it's weights have landed
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (gave_up) break;
        if (tid == 0) {
            if (TMA && !mbar_wait(smem_u32(&full[st]), (uint32_t)((it >> 1) & 1))) {
                gave_up = 1;
            } else {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t sa = smem_u32(base + st * kHStage), sb = sa + kHABytes;
                for (int tap = 0; tap < 27; ++tap) {
                    const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;  // halo row offsets
                    const uint64_t ad = tc_desc(sa + (uint32_t)(((dz * 3 + dy) * kHx + dx) * 16), kHPlanePad, 128);
                    const uint64_t bd = tc_desc(sb + (uint32_t)(tap * kTcN * 16), 27 * kTcN * 16, 128);
                    const uint32_t acc = (g == 0 && tap == 0) ? 0u : 1u;
                    asm volatile(
                        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                        :: "r"(tmem), "l"(ad), "l"(bd), "r"(kTcIdesc), "r"(acc) : "memory");
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                             :: "r"(smem_u32(&empty[st])) : "memory");
                if (g == G - 1)
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                                 :: "r"(smem_u32(&done)) : "memory");
            }
        }
        __syncthreads();
        if (gave_up) break;
        if (g == G - 1) {  // the tile's accumulator is complete: epilogue
            int z, yy, x0;
            tile_of(it, z, yy, x0);
            const bool ok = mbar_wait(smem_u32(&done), (uint32_t)(tiles_done & 1));
            ++tiles_done;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (!ok) {
                gave_up = 1;
            } else if (warp < 4) {  // warps 0-3 hold TMEM lanes 0-127, one output voxel per thread
                uint32_t r[32];
                const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                    "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
                      "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                      "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                    : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                const int x = x0 + tid;
                if (x < xa.w) {
                    const int64_t o = (((int64_t)z * xa.h + yy) * xa.w + x) * ya.cstride + ya.coff;
#pragma unroll
                    for (int j = 0; j < kTcN; j += 8) {
                        float f[8];
#pragma unroll
                        for (int e = 0; e < 8; ++e) {
                            const float t = __uint_as_float(r[j + e]) + (bias ? bias[j + e] : 0.0f);
                            f[e] = relu ? fmaxf(t, 0.0f) : t;
                        }
                        __nv_bfloat162 h[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) h[e] = __floats2bfloat162_rn(f[2 * e], f[2 * e + 1]);
                        *reinterpret_cast<uint4 *>(y + o + j) = *reinterpret_cast<const uint4 *>(h);
                        if (yf) {
#pragma unroll
                            for (int e = 0; e < 8; ++e) yf[o + j + e] = f[e];
                        }
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();  // the next tile's first MMA overwrites the accumulator
            if (gave_up) break;
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    if (gave_up) {
        if (tid == 0) {
            atomicExch(&g_tc_status, 1);
            // bounded waits for copies and MMAs that may still be in flight
            if (TMA) {
                mbar_wait(smem_u32(&full[0]), 0);
                mbar_wait(smem_u32(&full[1]), 0);
            }
            mbar_wait(smem_u32(&empty[0]), 0);
            mbar_wait(smem_u32(&empty[1]), 0);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kTcCols) : "memory");
}

// cuTensorMapEncodeTiled from the driver (the runtime is linked statically; no -lcuda)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

// Launches the halo kernel when the layer qualifies and its tensor maps encode; false otherwise
// (the caller then takes another kernel).
static bool launch_halo(const __nv_bfloat16 *x, const Act &xa, int cin, const __nv_bfloat16 *w, const float *bias,
                        int cout, int relu, __nv_bfloat16 *y, const Act &ya, float *yf, bool tma, cudaStream_t s) {
    if (xa.n != 1 || cout != kTcN || cin % 16 || cin / 8 > kHMaxChunks || xa.w < 96) return false;
    if (xa.cstride % 8 || xa.coff % 8 || ya.cstride % 8 || ya.coff % 8) return false;
    if ((uintptr_t)x % 16 || (uintptr_t)w % 16 || (uintptr_t)y % 16) return false;
    HaloMaps maps;
    memset(&maps, 0, sizeof(maps));
    if (tma) {
        EncodeTiledFn enc = encode_tiled();
        if (!enc) return false;
        const cuuint64_t dims[4] = {8, (cuuint64_t)xa.w, (cuuint64_t)xa.h, (cuuint64_t)xa.d};
        const cuuint64_t row = (cuuint64_t)xa.cstride * 2;
        const cuuint64_t strides[3] = {row, row * xa.w, row * xa.w * xa.h};
        const cuuint32_t box[4] = {8, (cuuint32_t)kHx, 3, 3};
        const cuuint32_t estr[4] = {1, 1, 1, 1};
        for (int c = 0; c < cin / 8; ++c) {
            void *addr = (void *)(x + xa.coff + 8 * c);
            if (enc(&maps.m[c], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, addr, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                return false;
        }
    }
    auto kern = tma ? k_conv3d_fwd_halo<true> : k_conv3d_fwd_halo<false>;
    static bool attr[2] = {false, false};
    if (!attr[tma]) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kHSmem) != cudaSuccess)
            return false;
        attr[tma] = true;
    }
    const int64_t n_tiles = (int64_t)xa.d * xa.h * ((xa.w + kTcM - 1) / kTcM);
    const unsigned grid = (unsigned)std::min<int64_t>(n_tiles, num_sms());
    kern<<<grid, 256, kHSmem, s>>>(maps, x, xa, cin, w, bias, relu, y, ya, yf);
    return true;
}



// Small grids (too few CTAs to hide the latency of a long chain of K steps): each of the 4 warps
// walks every 4th (tap, 16-channel) step of the whole 64-voxel x 32-channel tile through its own
// double buffer, synchronising only within the warp; the four partial tiles are then summed
// through shared memory (reusing the buffers) and written with the bias and activation.
constexpr int kWsM = 64, kWsN = 32, kWsRed = 36;  // reduction row stride (floats)
constexpr int kWsWarpBytes = (2 * kWsM + 2 * kWsN) * kCPad * 2;
static_assert(4 * kWsM * kWsRed * 4 <= 4 * kWsWarpBytes, "reduction fits in the staging buffers");

__global__ void __launch_bounds__(128)
k_conv3d_fwd_wsplit(const __nv_bfloat16 *__restrict__ x, Act xa, int cin, const __nv_bfloat16 *__restrict__ wt,
                    const float *__restrict__ bias, int cout, int relu, __nv_bfloat16 *__restrict__ y, Act ya,
                    float *__restrict__ yf) {
    __shared__ __align__(16) unsigned char smem[4 * kWsWarpBytes];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    typedef __nv_bfloat16 ARow[kCPad];
    ARow *As = reinterpret_cast<ARow *>(smem + warp * kWsWarpBytes);  // [2][kWsM]
    ARow *Bs = As + 2 * kWsM;                                          // [2][kWsN]
    const int64_t nvox = (int64_t)xa.d * xa.h * xa.w;
    const int64_t v0 = (int64_t)blockIdx.x * kWsM;
    const int co0 = blockIdx.y * kWsN;
    const int nb = blockIdx.z;
    const __nv_bfloat16 *xb = x + (int64_t)nb * nvox * xa.cstride + xa.coff;
    // lane slots: A rows lane / 2 + 16 i (i < 4), B rows lane / 2 + 16 i (i < 2), half (lane & 1) * 8
    const int lh = (lane & 1) * 8, r0 = lane >> 1;
    int lz[4], ly[4], lx[4];
    bool lok[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t v = v0 + r0 + 16 * i;
        lok[i] = v < nvox;
        const int z = lok[i] ? (int)(v / ((int64_t)xa.h * xa.w)) : 0;
        const int rem = lok[i] ? (int)(v - (int64_t)z * xa.h * xa.w) : 0;
        lz[i] = z;
        ly[i] = rem / xa.w;
        lx[i] = rem - ly[i] * xa.w;
    }
    uint4 ra[4], rb[2];
    const int nck = cin / kCK, steps = 27 * nck;
    auto load = [&](int st) {
        const int tap = st / nck, c0 = (st - tap * nck) * kCK;
        const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int zz = lz[i] + dz, yy = ly[i] + dy, xx = lx[i] + dx;
            const bool in = lok[i] && zz >= 0 && zz < xa.d && yy >= 0 && yy < xa.h && xx >= 0 && xx < xa.w;
            ra[i] = make_uint4(0, 0, 0, 0);
            if (in) ra[i] = *reinterpret_cast<const uint4 *>(xb + (((int64_t)zz * xa.h + yy) * xa.w + xx) * xa.cstride + c0 + lh);
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int co = co0 + r0 + 16 * i;
            rb[i] = make_uint4(0, 0, 0, 0);
            if (co < cout) rb[i] = *reinterpret_cast<const uint4 *>(wt + ((int64_t)co * 27 + tap) * cin + c0 + lh);
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int i = 0; i < 4; ++i) *reinterpret_cast<uint4 *>(&As[buf * kWsM + r0 + 16 * i][lh]) = ra[i];
#pragma unroll
        for (int i = 0; i < 2; ++i) *reinterpret_cast<uint4 *>(&Bs[buf * kWsN + r0 + 16 * i][lh]) = rb[i];
    };
    float acc[4][4][4] = {};
    if (warp < steps) {
        load(warp);
        store(0);
    }
    __syncwarp();
    int it = 0;
    for (int st = warp; st < steps; st += 4, ++it) {
        const int cur = it & 1;
        const bool more = st + 4 < steps;
        if (more) load(st + 4);
        warp_mma_tile<4, 4>(As + cur * kWsM, Bs + cur * kWsN, 0, acc);
        if (more) store(cur ^ 1);
        __syncwarp();
    }
    __syncthreads();  // every warp is done with its staging buffers
    float *red = reinterpret_cast<float *>(smem) + warp * kWsM * kWsRed;
    const int grp = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                const int r = m * 16 + grp + half * 8, c = j * 8 + tig * 2;
                *reinterpret_cast<float2 *>(&red[r * kWsRed + c]) =
                    make_float2(acc[m][j][half * 2], acc[m][j][half * 2 + 1]);
            }
    __syncthreads();
    // thread t: column pair t % 16, rows t / 16 + 8 k
    const float *red0 = reinterpret_cast<const float *>(smem);
    const int cp = (tid & 15) * 2, co = co0 + cp;
    if (co < cout) {
        const float b0 = bias ? bias[co] : 0.0f, b1 = bias ? bias[co + 1] : 0.0f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int r = (tid >> 4) + 8 * k;
            const int64_t v = v0 + r;
            if (v >= nvox) continue;
            float s0 = b0, s1 = b1;
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                const float2 p = *reinterpret_cast<const float2 *>(&red0[(w * kWsM + r) * kWsRed + cp]);
                s0 += p.x;
                s1 += p.y;
            }
            if (relu) {
                s0 = fmaxf(s0, 0.0f);
                s1 = fmaxf(s1, 0.0f);
            }
            const int64_t o = ((int64_t)nb * nvox + v) * ya.cstride + ya.coff + co;
            *reinterpret_cast<__nv_bfloat162 *>(y + o) = __floats2bfloat162_rn(s0, s1);
            if (yf) {
                yf[o] = s0;
                yf[o + 1] = s1;
            }
        }
    }
}

// dw[co, tap, ci] += sum_v dy[v, co] x[v + tap - 1, ci]; grid (voxel splits, 27 taps, co/ci tiles)
__global__ void __launch_bounds__(128)
k_conv3d_wgrad(const __nv_bfloat16 *__restrict__ x, Act xa, int cin, const __nv_bfloat16 *__restrict__ dy,
               Act da, int cout, float *__restrict__ dw, int64_t vox_per_split) {
    __shared__ __align__(16) __nv_bfloat16 As[kCM][kCPad];  // [co][v]
    __shared__ __align__(16) __nv_bfloat16 Bs[kCN][kCPad];  // [ci][v]
    const int64_t nvox = (int64_t)xa.d * xa.h * xa.w;
    const int64_t total = nvox * xa.n;
    const int tap = blockIdx.y;
    const int dz = tap / 9 - 1, dyo = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    const int ci_tiles = (cin + kCN - 1) / kCN;
    const int co0 = (blockIdx.z / ci_tiles) * kCM, ci0 = (blockIdx.z % ci_tiles) * kCN;
    const int64_t vbeg = (int64_t)blockIdx.x * vox_per_split;
    const int64_t vend = min(total, vbeg + vox_per_split);
    const int tid = threadIdx.x, warp = tid >> 5;
    float acc[8][4] = {};
    // loader role: thread t handles voxel (t & 15) of the chunk and an 8-channel group (t >> 4)
    const int lvv = tid & 15, lg = tid >> 4;  // lg in [0, 8): channels lg*8 .. lg*8+7
    for (int64_t vc = vbeg; vc < vend; vc += kCK) {
        const int64_t v = vc + lvv;
        __nv_bfloat16 da8[8], xa8[8];
        bool vok = v < vend;
        int64_t nb = 0, lv = 0;
        if (vok) {
            nb = v / nvox;
            lv = v - nb * nvox;
        }
        // dy row (v, co0 + lg*8 ..)
        {
            uint4 t = make_uint4(0, 0, 0, 0);
            if (vok && co0 + lg * 8 < cout)
                t = *reinterpret_cast<const uint4 *>(dy + (nb * nvox + lv) * da.cstride + da.coff + co0 + lg * 8);
            *reinterpret_cast<uint4 *>(da8) = t;
        }
        // shifted x row (v + tap - 1, ci0 + lg*8 ..)
        {
            uint4 t = make_uint4(0, 0, 0, 0);
            if (vok) {
                const int z = (int)(lv / ((int64_t)xa.h * xa.w));
                const int rem = (int)(lv - (int64_t)z * xa.h * xa.w);
                const int yy = rem / xa.w + dyo, xx = rem % xa.w + dx, zz = z + dz;
                if (zz >= 0 && zz < xa.d && yy >= 0 && yy < xa.h && xx >= 0 && xx < xa.w && ci0 + lg * 8 < cin)
                    t = *reinterpret_cast<const uint4 *>(
                        x + ((nb * nvox) + ((int64_t)zz * xa.h + yy) * xa.w + xx) * xa.cstride + xa.coff + ci0 + lg * 8);
            }
            *reinterpret_cast<uint4 *>(xa8) = t;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            As[lg * 8 + j][lvv] = da8[j];
            Bs[lg * 8 + j][lvv] = xa8[j];
        }
        __syncthreads();
        warp_mma_step(As, Bs, warp * 16, acc);
        __syncthreads();
    }
    const int lane = tid & 31, grp = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int ci = ci0 + j * 8 + tig * 2;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int co = co0 + warp * 16 + grp + half * 8;
            if (co >= cout || ci >= cin) continue;
            float *p = dw + ((int64_t)co * 27 + tap) * cin + ci;
            atomicAdd(p, acc[j][half * 2]);
            atomicAdd(p + 1, acc[j][half * 2 + 1]);
        }
    }
}

// wf[ci, tap, co] = w[co, 26 - tap, ci]: weights of the data-gradient convolution
__global__ void k_flip_weights(const __nv_bfloat16 *__restrict__ w, int cout, int cin,
                               __nv_bfloat16 *__restrict__ wf) {
    const int64_t total = (int64_t)cout * 27 * cin;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int ci = (int)(i % cin);
        const int tap = (int)((i / cin) % 27);
        const int co = (int)(i / ((int64_t)cin * 27));
        wf[((int64_t)ci * 27 + (26 - tap)) * cout + co] = w[i];
    }
}

// elementwise helpers over NDHWC slices
__global__ void k_relu_bwd(__nv_bfloat16 *__restrict__ g, Act ga, const __nv_bfloat16 *__restrict__ y, Act ya,
                           int c, int64_t nvox_total) {
    const int64_t total = nvox_total * c;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = i / c;
        const int ch = (int)(i - v * c);
        if (!(__bfloat162float(y[v * ya.cstride + ya.coff + ch]) > 0.0f))
            g[v * ga.cstride + ga.coff + ch] = __float2bfloat16(0.0f);
    }
}

__global__ void k_bias_grad(const __nv_bfloat16 *__restrict__ g, Act ga, int c, int64_t nvox_total,
                            float *__restrict__ db) {
    // one block per channel group of 32; threads stride over voxels
    const int ch = blockIdx.y * 32 + (threadIdx.x & 31);
    float s = 0.0f;
    if (ch < c)
        for (int64_t v = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); v < nvox_total; v += (int64_t)gridDim.x * (blockDim.x / 32))
            s += __bfloat162float(g[v * ga.cstride + ga.coff + ch]);
    if (ch < c) atomicAdd(db + ch, s);
}

// 2x2x2 average pooling and its transpose; nearest 2x upsampling and its transpose
// V consecutive channels as floats: 8 through one 16-byte access, or 1.
template <int V>
__device__ __forceinline__ void ld_ch(const __nv_bfloat16 *p, float (&f)[V]) {
    if constexpr (V == 8) {
        const uint4 u = *reinterpret_cast<const uint4 *>(p);
        const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float2 t = __bfloat1622float2(h[i]);
            f[2 * i] = t.x;
            f[2 * i + 1] = t.y;
        }
    } else {
        f[0] = __bfloat162float(*p);
    }
}

template <int V>
__device__ __forceinline__ void st_ch(__nv_bfloat16 *p, const float (&f)[V]) {
    if constexpr (V == 8) {
        uint4 u;
        __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&u);
#pragma unroll
        for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
        *reinterpret_cast<uint4 *>(p) = u;
    } else {
        *p = __float2bfloat16(f[0]);
    }
}

// Element i of a grid-stride loop over (voxel of `a`, group of V channels): the voxel's
// coordinates and the group's first channel.
struct VoxCh {
    int64_t nb;
    int z, y, x, ch;
};
__device__ __forceinline__ VoxCh vox_ch(int64_t i, const Act &a, int groups, int V) {
    VoxCh r;
    r.ch = (int)(i % groups) * V;
    int64_t v = i / groups;
    r.x = (int)(v % a.w);
    v /= a.w;
    r.y = (int)(v % a.h);
    v /= a.h;
    r.z = (int)(v % a.d);
    r.nb = v / a.d;
    return r;
}

__device__ __forceinline__ int64_t act_off(const Act &a, int64_t nb, int z, int y, int x, int ch) {
    return (((nb * a.d + z) * a.h + y) * a.w + x) * a.cstride + a.coff + ch;
}

// y (coarse) = mean of the 8 children in x (fine), children outside the fine grid counting 0
template <int V>
__global__ void k_avgpool2(const __nv_bfloat16 *__restrict__ x, Act xa, __nv_bfloat16 *__restrict__ y, Act ya, int c) {
    const int groups = c / V;
    const int64_t total = (int64_t)ya.n * ya.d * ya.h * ya.w * groups;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const VoxCh o = vox_ch(i, ya, groups, V);
        float s[V] = {};
        for (int k = 0; k < 8; ++k) {
            const int zz = 2 * o.z + (k >> 2), yy = 2 * o.y + ((k >> 1) & 1), xx = 2 * o.x + (k & 1);
            if (zz < xa.d && yy < xa.h && xx < xa.w) {
                float f[V];
                ld_ch<V>(x + act_off(xa, o.nb, zz, yy, xx, o.ch), f);
#pragma unroll
                for (int q = 0; q < V; ++q) s[q] += f[q];
            }
        }
#pragma unroll
        for (int q = 0; q < V; ++q) s[q] *= 0.125f;
        st_ch<V>(y + act_off(ya, o.nb, o.z, o.y, o.x, o.ch), s);
    }
}

// dx (fine) = dy (coarse) / 8 for the 8 children (the adjoint of k_avgpool2)
template <int V>
__global__ void k_avgpool2_bwd(const __nv_bfloat16 *__restrict__ dy, Act ya, __nv_bfloat16 *__restrict__ dx, Act xa, int c) {
    const int groups = c / V;
    const int64_t total = (int64_t)xa.n * xa.d * xa.h * xa.w * groups;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const VoxCh f = vox_ch(i, xa, groups, V);
        const int oz = f.z / 2, oy = f.y / 2, ox = f.x / 2;
        float g[V] = {};
        if (oz < ya.d && oy < ya.h && ox < ya.w) {
            ld_ch<V>(dy + act_off(ya, f.nb, oz, oy, ox, f.ch), g);
#pragma unroll
            for (int q = 0; q < V; ++q) g[q] *= 0.125f;
        }
        st_ch<V>(dx + act_off(xa, f.nb, f.z, f.y, f.x, f.ch), g);
    }
}

// y (fine) = x (coarse) at the parent voxel; mode 1: the adjoint (sum of the 8 children)
template <int V>
__global__ void k_upsample2(const __nv_bfloat16 *__restrict__ src, Act sa, __nv_bfloat16 *__restrict__ dst, Act da,
                            int c, int adjoint) {
    const int groups = c / V;
    const int64_t total = (int64_t)da.n * da.d * da.h * da.w * groups;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const VoxCh o = vox_ch(i, da, groups, V);
        float r[V] = {};
        if (!adjoint) {  // dst fine, src coarse
            ld_ch<V>(src + act_off(sa, o.nb, o.z / 2, o.y / 2, o.x / 2, o.ch), r);
        } else {  // dst coarse, src fine
            for (int k = 0; k < 8; ++k) {
                const int zz = 2 * o.z + (k >> 2), yy = 2 * o.y + ((k >> 1) & 1), xx = 2 * o.x + (k & 1);
                if (zz < sa.d && yy < sa.h && xx < sa.w) {
                    float f[V];
                    ld_ch<V>(src + act_off(sa, o.nb, zz, yy, xx, o.ch), f);
#pragma unroll
                    for (int q = 0; q < V; ++q) r[q] += f[q];
                }
            }
        }
        st_ch<V>(dst + act_off(da, o.nb, o.z, o.y, o.x, o.ch), r);
    }
}

// Sub-voxel head: 8 FP32 outputs per coarse voxel v = (z, y, x), output q = 4i + 2j + k landing at
// fine voxel (2z + i, 2y + j, 2x + k) of an (n, D, H, W) grid (outputs past D/H/W are dropped):
// out = b[q] + sum_c x[v, c] w[q][c]. Weights [8][c] FP32, c <= 64. Voxel counts are below 2^31
// (checked on the host), so the index arithmetic is 32-bit.
struct Fine {
    int64_t base;      // fine offset of sub-voxel (0, 0, 0)
    int lim;           // bit q set when sub-voxel q lies inside the fine grid
};

__device__ __forceinline__ Fine fine_of(int v, const Act &xa, int D, int H, int W) {
    int r = v;
    const int x = r % xa.w; r /= xa.w;
    const int y = r % xa.h; r /= xa.h;
    const int z = r % xa.d;
    const int nb = r / xa.d;
    Fine f;
    f.base = (((int64_t)nb * D + 2 * z) * H + 2 * y) * (int64_t)W + 2 * x;
    const bool zi = 2 * z + 1 < D, yi = 2 * y + 1 < H, xi = 2 * x + 1 < W;
    f.lim = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q)
        if ((!(q & 4) || zi) && (!(q & 2) || yi) && (!(q & 1) || xi)) f.lim |= 1 << q;
    return f;
}

__device__ __forceinline__ int64_t fine_off(const Fine &f, int q, int H, int W) {
    return f.base + ((int64_t)(q >> 2) * H + ((q >> 1) & 1)) * W + (q & 1);
}

__global__ void k_head8_fwd(const __nv_bfloat16 *__restrict__ x, Act xa, int c, const float *__restrict__ w,
                            const float *__restrict__ bp, float *__restrict__ out, int D, int H, int W,
                            int nvox_total) {
    __shared__ float sw[8][64];
    __shared__ float sb[8];
    for (int t = threadIdx.x; t < 8 * 64; t += blockDim.x) sw[t >> 6][t & 63] = (t & 63) < c ? w[(t >> 6) * c + (t & 63)] : 0.0f;
    if (threadIdx.x < 8) sb[threadIdx.x] = bp ? bp[threadIdx.x] : 0.0f;
    __syncthreads();
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nvox_total; v += gridDim.x * blockDim.x) {
        float acc[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[q] = sb[q];
        const __nv_bfloat16 *xr = x + (int64_t)v * xa.cstride + xa.coff;
        for (int ch = 0; ch < c; ++ch) {
            const float xv = __bfloat162float(xr[ch]);
#pragma unroll
            for (int q = 0; q < 8; ++q) acc[q] = fmaf(xv, sw[q][ch], acc[q]);
        }
        const Fine f = fine_of(v, xa, D, H, W);
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (f.lim >> q & 1) out[fine_off(f, q, H, W)] = acc[q];
    }
}

// gx[v, ch] = sum_q gout[fine(v, q)] w[q][ch]; one thread per (voxel, channel)
__global__ void k_head8_dx(const float *__restrict__ gout, Act xa, int c, const float *__restrict__ w,
                           __nv_bfloat16 *__restrict__ gx, Act ga, int D, int H, int W, int64_t total) {
    __shared__ float sw[8][64];
    for (int t = threadIdx.x; t < 8 * 64; t += blockDim.x) sw[t >> 6][t & 63] = (t & 63) < c ? w[(t >> 6) * c + (t & 63)] : 0.0f;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int v = (int)(i / c);
        const int ch = (int)(i - (int64_t)v * c);
        const Fine f = fine_of(v, xa, D, H, W);
        float s = 0.0f;
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (f.lim >> q & 1) s = fmaf(gout[fine_off(f, q, H, W)], sw[q][ch], s);
        gx[(int64_t)v * ga.cstride + ga.coff + ch] = __float2bfloat16(s);
    }
}

// gw[q][ch] += sum_v gout[fine(v, q)] x[v, ch], gb[q] += sum_v gout[fine(v, q)]. A block takes
// `chunk` voxels: their 8 sub-voxel gradients are staged in shared memory, then thread t owns
// the pairs (q, ch) = divmod(t + k * blockDim, c + 1) (ch == c is the bias) and adds one atomic
// per pair.
constexpr int kHeadChunk = 128;

__global__ void k_head8_dw(const __nv_bfloat16 *__restrict__ x, Act xa, int c, const float *__restrict__ gout,
                           float *__restrict__ gw, float *__restrict__ gb, int D, int H, int W, int nvox_total) {
    __shared__ float sg[kHeadChunk][8];
    const int v0 = blockIdx.x * kHeadChunk;
    const int nv = min(kHeadChunk, nvox_total - v0);
    for (int t = threadIdx.x; t < kHeadChunk * 8; t += blockDim.x) {
        const int j = t >> 3, q = t & 7;
        float g = 0.0f;
        if (j < nv) {
            const Fine f = fine_of(v0 + j, xa, D, H, W);
            if (f.lim >> q & 1) g = gout[fine_off(f, q, H, W)];
        }
        sg[j][q] = g;
    }
    __syncthreads();
    const int pairs = 8 * (c + 1);
    for (int t = threadIdx.x; t < pairs; t += blockDim.x) {
        const int q = t / (c + 1), ch = t - q * (c + 1);
        float s = 0.0f;
        if (ch < c) {
            const __nv_bfloat16 *xr = x + (int64_t)v0 * xa.cstride + xa.coff + ch;
            for (int j = 0; j < nv; ++j) s = fmaf(sg[j][q], __bfloat162float(xr[(int64_t)j * xa.cstride]), s);
            atomicAdd(gw + q * c + ch, s);
        } else {
            for (int j = 0; j < nv; ++j) s += sg[j][q];
            atomicAdd(gb + q, s);
        }
    }
}

// Adam on FP32 masters, refreshed BF16 copy (bf may be NULL for FP32-only parameters)
__global__ void k_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                       const float *__restrict__ g, __nv_bfloat16 *__restrict__ bf, int64_t n,
                       float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        if (bf) bf[i] = __float2bfloat16(wi);
    }
}

// dst slice += src slice (gradients of a tensor used twice, e.g. a U-Net skip)
__global__ void k_add(__nv_bfloat16 *__restrict__ dst, Act da, const __nv_bfloat16 *__restrict__ src, Act sa,
                      int c, int64_t nvox_total) {
    const int64_t total = nvox_total * c;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = i / c;
        const int ch = (int)(i - v * c);
        __nv_bfloat16 *d = dst + v * da.cstride + da.coff + ch;
        *d = __float2bfloat16(__bfloat162float(*d) + __bfloat162float(src[v * sa.cstride + sa.coff + ch]));
    }
}

// relative squared error per sample: loss += sum m (p - t)^2 * inv_den[s]; grad = 2 m (p - t) inv_den[s] / n_samples
__global__ void k_rel_mse(const float *__restrict__ pred, const float *__restrict__ target,
                          const float *__restrict__ mask, const float *__restrict__ inv_den, int64_t per_sample,
                          int n_samples, float *__restrict__ grad, double *__restrict__ loss) {
    double acc = 0.0;
    const int64_t total = per_sample * n_samples;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(i / per_sample);
        const float m = mask ? mask[i - (int64_t)s * per_sample] : 1.0f;
        const float d = pred[i] - target[i];
        acc += (double)(m * d * d) * (double)inv_den[s] / (double)n_samples;
        if (grad) grad[i] = 2.0f * m * d * inv_den[s] / (float)n_samples;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc != 0.0) atomicAdd(loss, acc);
}

inline int check_act(const Act &a, int c, const char *name) {
    if (a.n <= 0 || a.d <= 0 || a.h <= 0 || a.w <= 0) return fail(SRF_EGRID, "%s: bad shape", name);
    if (a.cstride < c + a.coff || a.coff < 0) return fail(SRF_EGRID, "%s: channel slice exceeds stride", name);
    if ((int64_t)a.n * a.d * a.h * a.w * a.cstride >= (int64_t(1) << 40)) return fail(SRF_ERANGE, "%s: too large", name);
    return SRF_OK;
}

inline Act act_of(const int32_t s[6]) { return Act{s[0], s[1], s[2], s[3], s[4], s[5]}; }

// Both channel slices hold whole 16-byte groups of 8 channels (16-byte aligned buffers and
// element offsets).
inline bool vec8(const void *pa, const Act &a, const void *pb, const Act &b, int c) {
    return c % 8 == 0 && a.cstride % 8 == 0 && a.coff % 8 == 0 && b.cstride % 8 == 0 && b.coff % 8 == 0 &&
           (uintptr_t)pa % 16 == 0 && (uintptr_t)pb % 16 == 0;
}

}  // namespace srf

using namespace srf;

extern "C" {

int srf_conv3d_fwd(const void *x, const int32_t xs[6], int32_t cin, const void *w, const float *bias,
                   int32_t cout, int32_t relu, void *y, const int32_t ys[6], float *yf, void *stream) {
    if (!x || !xs || !w || !y || !ys) return fail(SRF_EINVAL, "NULL argument");
    const Act xa = act_of(xs), ya = act_of(ys);
    int rc;
    if ((rc = check_act(xa, cin, "x")) || (rc = check_act(ya, cout, "y"))) return rc;
    if (cin % 16 || cout % 16 || xa.cstride % 8 || xa.coff % 8 || ya.cstride % 2 || ya.coff % 2)
        return fail(SRF_EINVAL, "conv3d needs Cin, Cout multiples of 16 and 16-byte aligned channel slices");
    if (xa.n != ya.n || xa.d != ya.d || xa.h != ya.h || xa.w != ya.w) return fail(SRF_EGRID, "x/y shapes differ");
    const int64_t nvox = (int64_t)xa.d * xa.h * xa.w;
    // the widest tile that still gives every SM two CTAs: 64 x 64 when Cout is a multiple of 64,
    // else 128 voxels x 32 channels (no idle columns at Cout = 32 or 96); below that, 64 x 32
    // tiles with K split over each CTA's warps
    const int64_t fill = 2 * (int64_t)num_sms();
    const auto ctas = [&](int bm, int bn) { return ((nvox + bm - 1) / bm) * ((cout + bn - 1) / bn) * xa.n; };
    const __nv_bfloat16 *xp = (const __nv_bfloat16 *)x, *wp = (const __nv_bfloat16 *)w;
    __nv_bfloat16 *yp = (__nv_bfloat16 *)y;
    const cudaStream_t s = (cudaStream_t)stream;
    if (cout % 64 == 0 && ctas(64, 64) >= fill) {
        dim3 grid((unsigned)((nvox + 63) / 64), (unsigned)(cout / 64), (unsigned)xa.n);
        k_conv3d_fwd<64, 64><<<grid, 128, 0, s>>>(xp, xa, cin, wp, bias, cout, relu, yp, ya, yf);
        g_conv_path = 0;
    } else if (g_conv_tc >= 2 && launch_halo(xp, xa, cin, wp, bias, cout, relu, yp, ya, yf, g_conv_tc == 3, s)) {
        g_conv_path = g_conv_tc == 3 ? 3 : 5;  // batch-1 wide layers: tcgen05 on halo tiles
    } else if (ctas(128, 32) >= fill) {
        dim3 grid((unsigned)((nvox + 127) / 128), (unsigned)((cout + 31) / 32), (unsigned)xa.n);
        if (g_conv_tc && cout % 32 == 0 && ya.cstride % 8 == 0 && ya.coff % 8 == 0 && (uintptr_t)y % 16 == 0 &&
            (uintptr_t)x % 16 == 0 && (uintptr_t)w % 16 == 0) {
            k_conv3d_fwd_tc<<<grid, 128, 0, s>>>(xp, xa, cin, wp, bias, cout, relu, yp, ya, yf);
            g_conv_path = 2;
        } else {
            k_conv3d_fwd<128, 32><<<grid, 128, 0, s>>>(xp, xa, cin, wp, bias, cout, relu, yp, ya, yf);
            g_conv_path = 1;
        }
    } else {  // too few CTAs to hide a long K chain: split K over the warps of each CTA
        dim3 grid((unsigned)((nvox + kWsM - 1) / kWsM), (unsigned)((cout + kWsN - 1) / kWsN), (unsigned)xa.n);
        k_conv3d_fwd_wsplit<<<grid, 128, 0, s>>>(xp, xa, cin, wp, bias, cout, relu, yp, ya, yf);
        g_conv_path = 4;
    }
    return check_cuda("conv3d forward launch");
}

int srf_set_conv_tc(int32_t mode) {
    if (mode < 0 || mode > 3) return fail(SRF_EINVAL, "conv mode must be 0, 1, 2 or 3");
    g_conv_tc = mode;
    return ok();
}

int srf_conv_last_path(int32_t *path) {
    if (!path) return fail(SRF_EINVAL, "NULL argument");
    *path = g_conv_path;
    return ok();
}

int srf_conv_tc_status(int32_t *status) {
    if (!status) return fail(SRF_EINVAL, "NULL argument");
    int h = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&h, g_tc_status, sizeof(int));
    if (e != cudaSuccess) return check_cuda("conv tc status");
    *status = h;
    return ok();
}

int srf_conv3d_wgrad(const void *x, const int32_t xs[6], int32_t cin, const void *dy, const int32_t ds[6],
                     int32_t cout, float *dw, void *stream) {
    if (!x || !xs || !dy || !ds || !dw) return fail(SRF_EINVAL, "NULL argument");
    const Act xa = act_of(xs), da = act_of(ds);
    int rc;
    if ((rc = check_act(xa, cin, "x")) || (rc = check_act(da, cout, "dy"))) return rc;
    if (cin % 16 || cout % 16 || xa.cstride % 8 || xa.coff % 8 || da.cstride % 8 || da.coff % 8)
        return fail(SRF_EINVAL, "conv3d needs Cin, Cout multiples of 16 and 16-byte aligned channel slices");
    const int64_t total = (int64_t)xa.n * xa.d * xa.h * xa.w;
    const int tiles = ((cout + kCM - 1) / kCM) * ((cin + kCN - 1) / kCN);
    // enough splits to fill the GPU: ~4 CTAs per SM over 27 taps x tiles
    int64_t want = (int64_t)num_sms() * 8 / (27 * tiles) + 1;
    int64_t per = (total + want - 1) / want;
    per = ((per + kCK - 1) / kCK) * kCK;
    const int64_t splits = (total + per - 1) / per;
    dim3 grid((unsigned)splits, 27, (unsigned)tiles);
    k_conv3d_wgrad<<<grid, 128, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)x, xa, cin, (const __nv_bfloat16 *)dy,
                                                          da, cout, dw, per);
    return check_cuda("conv3d weight-gradient launch");
}

int srf_conv3d_flip_weights(const void *w, int32_t cout, int32_t cin, void *wf, void *stream) {
    if (!w || !wf || cout <= 0 || cin <= 0) return fail(SRF_EINVAL, "bad arguments");
    const int64_t total = (int64_t)cout * 27 * cin;
    k_flip_weights<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16 *)w, cout, cin, (__nv_bfloat16 *)wf);
    return check_cuda("flip weights launch");
}

int srf_cnn_relu_bwd(void *g, const int32_t gs[6], const void *y, const int32_t ys[6], int32_t c, void *stream) {
    const Act ga = act_of(gs), ya = act_of(ys);
    int rc;
    if ((rc = check_act(ga, c, "g")) || (rc = check_act(ya, c, "y"))) return rc;
    const int64_t nv = (int64_t)ga.n * ga.d * ga.h * ga.w;
    unsigned blocks = grid_for(k_relu_bwd, nv * c, 256);
    k_relu_bwd<<<blocks, 256, 0, (cudaStream_t)stream>>>((__nv_bfloat16 *)g, ga, (const __nv_bfloat16 *)y, ya, c, nv);
    return check_cuda("relu backward launch");
}

int srf_cnn_bias_grad(const void *g, const int32_t gs[6], int32_t c, float *db, void *stream) {
    const Act ga = act_of(gs);
    int rc;
    if ((rc = check_act(ga, c, "g"))) return rc;
    const int64_t nv = (int64_t)ga.n * ga.d * ga.h * ga.w;
    dim3 grid((unsigned)std::min<int64_t>(1024, (nv + 7) / 8), (unsigned)((c + 31) / 32));
    k_bias_grad<<<grid, 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)g, ga, c, nv, db);
    return check_cuda("bias gradient launch");
}

int srf_cnn_pool2(const void *x, const int32_t xs[6], void *y, const int32_t ys[6], int32_t c, int32_t adjoint,
                  void *stream) {
    const Act xa = act_of(xs), ya = act_of(ys);  // x fine, y coarse
    int rc;
    if ((rc = check_act(xa, c, "fine")) || (rc = check_act(ya, c, "coarse"))) return rc;
    if (ya.d != (xa.d + 1) / 2 || ya.h != (xa.h + 1) / 2 || ya.w != (xa.w + 1) / 2 || xa.n != ya.n)
        return fail(SRF_EGRID, "coarse grid must be ceil(fine / 2)");
    cudaStream_t s = (cudaStream_t)stream;
    const __nv_bfloat16 *xc = (const __nv_bfloat16 *)x, *yc = (const __nv_bfloat16 *)y;
    __nv_bfloat16 *xm = (__nv_bfloat16 *)x, *ym = (__nv_bfloat16 *)y;
    if (vec8(x, xa, y, ya, c)) {
        if (!adjoint) {
            const int64_t t = (int64_t)ya.n * ya.d * ya.h * ya.w * (c / 8);
            k_avgpool2<8><<<grid_for(k_avgpool2<8>, t, 256), 256, 0, s>>>(xc, xa, ym, ya, c);
        } else {
            const int64_t t = (int64_t)xa.n * xa.d * xa.h * xa.w * (c / 8);
            k_avgpool2_bwd<8><<<grid_for(k_avgpool2_bwd<8>, t, 256), 256, 0, s>>>(yc, ya, xm, xa, c);
        }
    } else if (!adjoint) {
        const int64_t t = (int64_t)ya.n * ya.d * ya.h * ya.w * c;
        k_avgpool2<1><<<grid_for(k_avgpool2<1>, t, 256), 256, 0, s>>>(xc, xa, ym, ya, c);
    } else {  // y holds the coarse gradient, x receives the fine gradient
        const int64_t t = (int64_t)xa.n * xa.d * xa.h * xa.w * c;
        k_avgpool2_bwd<1><<<grid_for(k_avgpool2_bwd<1>, t, 256), 256, 0, s>>>(yc, ya, xm, xa, c);
    }
    return check_cuda("pool launch");
}

int srf_cnn_upsample2(const void *coarse, const int32_t cs[6], void *fine, const int32_t fs[6], int32_t c,
                      int32_t adjoint, void *stream) {
    const Act ca = act_of(cs), fa = act_of(fs);
    int rc;
    if ((rc = check_act(ca, c, "coarse")) || (rc = check_act(fa, c, "fine"))) return rc;
    if (ca.d != (fa.d + 1) / 2 || ca.h != (fa.h + 1) / 2 || ca.w != (fa.w + 1) / 2 || ca.n != fa.n)
        return fail(SRF_EGRID, "coarse grid must be ceil(fine / 2)");
    cudaStream_t s = (cudaStream_t)stream;
    const __nv_bfloat16 *cc = (const __nv_bfloat16 *)coarse, *fc = (const __nv_bfloat16 *)fine;
    __nv_bfloat16 *cm = (__nv_bfloat16 *)coarse, *fm = (__nv_bfloat16 *)fine;
    const bool v8 = vec8(coarse, ca, fine, fa, c);
    if (!adjoint) {
        const int64_t t = (int64_t)fa.n * fa.d * fa.h * fa.w * c;
        if (v8)
            k_upsample2<8><<<grid_for(k_upsample2<8>, t / 8, 256), 256, 0, s>>>(cc, ca, fm, fa, c, 0);
        else
            k_upsample2<1><<<grid_for(k_upsample2<1>, t, 256), 256, 0, s>>>(cc, ca, fm, fa, c, 0);
    } else {  // fine holds the gradient, coarse receives the sum over children
        const int64_t t = (int64_t)ca.n * ca.d * ca.h * ca.w * c;
        if (v8)
            k_upsample2<8><<<grid_for(k_upsample2<8>, t / 8, 256), 256, 0, s>>>(fc, fa, cm, ca, c, 1);
        else
            k_upsample2<1><<<grid_for(k_upsample2<1>, t, 256), 256, 0, s>>>(fc, fa, cm, ca, c, 1);
    }
    return check_cuda("upsample launch");
}

int srf_cnn_head8(const void *x, const int32_t xs[6], int32_t c, const float *w, const float *b, float *out,
                  const int32_t fine[3], const float *gout, void *gx, const int32_t gs[6], float *gw,
                  float *gb, void *stream) {
    if (c <= 0 || c > 64) return fail(SRF_EINVAL, "head supports 1..64 channels");
    if (!x || !xs || !w || !fine) return fail(SRF_EINVAL, "x, xs, w and fine must not be NULL");
    const Act xa = act_of(xs);
    int rc;
    if ((rc = check_act(xa, c, "x"))) return rc;
    const int D = fine[0], H = fine[1], W = fine[2];
    if (D <= 0 || H <= 0 || W <= 0 || D > 2 * xa.d || H > 2 * xa.h || W > 2 * xa.w)
        return fail(SRF_EGRID, "fine grid must be within twice the coarse grid");
    const int64_t nv = (int64_t)xa.n * xa.d * xa.h * xa.w;
    if (nv >= (int64_t(1) << 31)) return fail(SRF_ERANGE, "head8 supports fewer than 2^31 voxels");
    cudaStream_t s = (cudaStream_t)stream;
    if (!gout) {
        if (!out) return fail(SRF_EINVAL, "out must not be NULL");
        k_head8_fwd<<<grid_for(k_head8_fwd, nv, 256), 256, 0, s>>>((const __nv_bfloat16 *)x, xa, c, w, b, out, D, H, W, (int)nv);
        return check_cuda("head8 launch");
    }
    if (gx) {
        const Act ga = act_of(gs);
        if ((rc = check_act(ga, c, "gx"))) return rc;
        if (ga.n != xa.n || ga.d != xa.d || ga.h != xa.h || ga.w != xa.w) return fail(SRF_EGRID, "gx shape differs from x");
        k_head8_dx<<<grid_for(k_head8_dx, nv * c, 256), 256, 0, s>>>(gout, xa, c, w, (__nv_bfloat16 *)gx, ga, D, H, W, nv * c);
    }
    if (gw && gb) {
        const int64_t blocks = (nv + kHeadChunk - 1) / kHeadChunk;
        k_head8_dw<<<(unsigned)blocks, 288, 0, s>>>((const __nv_bfloat16 *)x, xa, c, gout, gw, gb, D, H, W, (int)nv);
    }
    return check_cuda("head8 gradient launch");
}

int srf_cnn_add(void *dst, const int32_t ds[6], const void *src, const int32_t ss[6], int32_t c, void *stream) {
    const Act da = act_of(ds), sa = act_of(ss);
    int rc;
    if ((rc = check_act(da, c, "dst")) || (rc = check_act(sa, c, "src"))) return rc;
    const int64_t nv = (int64_t)da.n * da.d * da.h * da.w;
    k_add<<<grid_for(k_add, nv * c, 256), 256, 0, (cudaStream_t)stream>>>((__nv_bfloat16 *)dst, da,
                                                                         (const __nv_bfloat16 *)src, sa, c, nv);
    return check_cuda("add launch");
}

int srf_cnn_rel_mse(const float *pred, const float *target, const float *mask, const float *inv_den,
                    int64_t per_sample, int32_t n_samples, float *grad, double *loss, void *stream) {
    if (!pred || !target || !inv_den || !loss || per_sample <= 0 || n_samples <= 0) return fail(SRF_EINVAL, "bad arguments");
    k_rel_mse<<<grid_for(k_rel_mse, per_sample * n_samples, 256), 256, 0, (cudaStream_t)stream>>>(
        pred, target, mask, inv_den, per_sample, n_samples, grad, loss);
    return check_cuda("loss launch");
}

int srf_cnn_adam(float *w, float *m, float *v, const float *g, void *bf16_copy, int64_t n, float lr,
                 float b1, float b2, float eps, int32_t step, void *stream) {
    if (!w || !m || !v || !g || n < 0 || step < 1) return fail(SRF_EINVAL, "bad arguments");
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    k_adam<<<grid_for(k_adam, n, 256), 256, 0, (cudaStream_t)stream>>>(w, m, v, g, (__nv_bfloat16 *)bf16_copy, n,
                                                                       lr, b1, b2, eps, c1, c2);
    return check_cuda("adam launch");
}

}  // extern "C"
