// sg4_items.cu -- the persistent H.psi kernels of one launch geometry.
// Compiled once per geometry (EVR_GEO = 0 wide, 1 narrow, 2 mid), in
// parallel, so each translation unit instantiates one pair of kernels; the
// host code in sg4_device.cu reaches them through the GeoKernels tables.
#include "sg4_items.cuh"

#ifndef EVR_GEO
#error "compile with -DEVR_GEO=0 (wide), 1 (narrow) or 2 (mid)"
#endif

namespace evr {

#if EVR_GEO == 0
#define EVR_G_CTAS EVR_WIDE_CTAS
#define EVR_G_FMAX EVR_WIDE_FMAX
#define EVR_G_TABLE geo_kernels_wide
#elif EVR_GEO == 1
#define EVR_G_CTAS EVR_NARROW_CTAS
#define EVR_G_FMAX EVR_NARROW_FMAX
#define EVR_G_TABLE geo_kernels_narrow
#else
#define EVR_G_CTAS EVR_MID_CTAS
#define EVR_G_FMAX EVR_MID_FMAX
#define EVR_G_TABLE geo_kernels_mid
#endif

static void g_batched(unsigned grid, size_t smem, cudaStream_t s, const KParams& p) {
  hpsi_batched_kernel<EVR_G_CTAS, EVR_G_FMAX><<<grid, EVR_CTA_THREADS, smem, s>>>(p);
}

static void g_multi(unsigned grid, size_t smem, cudaStream_t s, const KParams* ps, const MItem* items, int n_items,
                    int item_base, unsigned int* counter) {
  hpsi_multi_kernel<EVR_G_CTAS, EVR_G_FMAX><<<grid, EVR_CTA_THREADS, smem, s>>>(ps, items, n_items, item_base, counter);
}

static cudaError_t g_static_smem(size_t* batched, size_t* multi) {
  cudaFuncAttributes a, b;
  cudaError_t e = cudaFuncGetAttributes(&a, hpsi_batched_kernel<EVR_G_CTAS, EVR_G_FMAX>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&b, hpsi_multi_kernel<EVR_G_CTAS, EVR_G_FMAX>);
  if (e != cudaSuccess) return e;
  *batched = a.sharedSizeBytes;
  *multi = b.sharedSizeBytes;
  return cudaSuccess;
}

static cudaError_t g_set_smem(int bytes) {
  cudaError_t e = cudaFuncSetAttribute(hpsi_batched_kernel<EVR_G_CTAS, EVR_G_FMAX>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(hpsi_multi_kernel<EVR_G_CTAS, EVR_G_FMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             bytes);
  return e;
}

const GeoKernels EVR_G_TABLE = {EVR_G_CTAS, g_batched, g_multi, g_static_smem, g_set_smem};

}  // namespace evr
