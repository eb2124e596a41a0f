// Sensitivity image over all ordered crystal pairs, with the LORs generated on the device.
//
// srfnef's EcatEmapGenerator('block-full') (srfnef/functions/emap_generator.py:77-111) builds, for
// each of nb x nb block columns, an M^2-row LOR array on the host with numpy and launches the
// non-TOF backprojector on it (2304 launches and 1.05e9 LORs for a 48-block, 676-crystal-column
// scanner). Here LOR k = ((i*nb + j)*M + a)*M + b takes endpoint 1 from table row i*M + a and
// endpoint 2 from row j*M + b of a crystal table that holds exactly the float32 positions the
// reference computes (srf_gb300.geometry.block_full_crystal_table), and every LOR goes through
// the backprojector traversal with value 1.
#include "common.cuh"

namespace srf {

template <int G>
__global__ void __launch_bounds__(kBlock)
k_emap(const float *__restrict__ table, int nb, int m, Grid g, View v, View vt) {
    constexpr int GPW = 32 / G;
    const int lane = threadIdx.x & (G - 1);
    const int gi = (threadIdx.x & 31) / G;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t mm = (int64_t)m * m;
    const int64_t n = (int64_t)nb * nb * mm;
    const bool have_t = vt.ptr != nullptr;
    const TofParams tp{0, 0, 0};
    for (int64_t base = warp * GPW; base < n; base += nwarps * GPW) {
        const int64_t k = base + gi;
        if (k >= n) continue;
        const int64_t blk = k / mm, rem = k - blk * mm;
        const int i = (int)(blk / nb), j = (int)(blk - (int64_t)(blk / nb) * nb);
        const int a = (int)(rem / m), b = (int)(rem - (int64_t)(rem / m) * m);
        const float *e1 = table + 3 * ((int64_t)i * m + a);
        const float *e2 = table + 3 * ((int64_t)j * m + b);
        LorSetup S;
        if (setup_lor<false, RULES_BACK>(__ldg(e1), __ldg(e1 + 1), __ldg(e1 + 2), __ldg(e2),
                                         __ldg(e2 + 1), __ldg(e2 + 2), 0.0f, g, tp, v.st, vt.st,
                                         have_t, S)) {
            float *im = (!S.xdom && have_t) ? vt.ptr : v.ptr;
            for (int ip = S.lo + lane; ip <= S.hi; ip += G)
                slab<false, RULES_BACK>(S, ip, [&](int32_t off, float w) { atomicAdd(im + off, w); });
        }
    }
}

}  // namespace srf

using namespace srf;

extern "C" int srf_emap_block_full(const float *crystal_table, int32_t n_blocks, int32_t m,
                                   float *emap, const int64_t emap_strides[3], float *emap_t,
                                   const int64_t emap_t_strides[3], const int32_t grid[3],
                                   const float center[3], const float size[3], void *stream) {
    Grid g; View v, vt; int rc;
    if (!crystal_table) return fail(SRF_EINVAL, "crystal_table must not be NULL");
    if (n_blocks <= 0 || m <= 0) return fail(SRF_EINVAL, "n_blocks and m must be positive");
    if ((rc = check_geometry(grid, center, size, g))) return rc;
    if ((rc = check_view(emap, emap_strides, g, "emap", v, true))) return rc;
    if ((rc = check_view(emap_t, emap_t_strides, g, "emap_t", vt, false))) return rc;
    const int64_t n = (int64_t)n_blocks * n_blocks * (int64_t)m * m;
    cudaStream_t s = (cudaStream_t)stream;
    switch (group_lanes()) {
    case 8: { auto k = k_emap<8>; k<<<grid_for(k, n, kBlock / 8), kBlock, 0, s>>>(crystal_table, n_blocks, m, g, v, vt); break; }
    case 16: { auto k = k_emap<16>; k<<<grid_for(k, n, kBlock / 16), kBlock, 0, s>>>(crystal_table, n_blocks, m, g, v, vt); break; }
    default: { auto k = k_emap<32>; k<<<grid_for(k, n, kBlock / 32), kBlock, 0, s>>>(crystal_table, n_blocks, m, g, v, vt); break; }
    }
    return check_cuda("emap kernel launch");
}
