// Sensitivity image over all ordered crystal pairs, with the LORs generated on the device.
//
// srfnef's EcatEmapGenerator('block-full') (srfnef/functions/emap_generator.py:77-111) builds, for
// each of nb x nb block columns, an M^2-row LOR array on the host with numpy and launches the
// non-TOF backprojector on it (2304 launches and 1.05e9 LORs for a 48-block, 676-crystal-column
// scanner). Here LOR k = ((i*nb + j)*M + a)*M + b takes endpoint 1 from table row i*M + a and
// endpoint 2 from row j*M + b of a crystal table that holds exactly the float32 positions the
// reference computes (srf_gb300.geometry.block_full_crystal_table), and every LOR goes through
// the fused kernel's backprojector traversal with value 1 (k_emap_fused in osem.cu).
#include "common.cuh"
#include "fused.cuh"

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
    return fused_emap(crystal_table, n_blocks, m, g, v, vt, (cudaStream_t)stream);
}
