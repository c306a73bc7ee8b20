// sg4_items.cu -- the persistent H.psi kernel of one launch geometry and one
// parameter-block size.  Compiled once per (geometry, kind), in parallel:
// EVR_GEO = 0 wide, 1 narrow, 2 mid; EVR_KIND = 0 the small block (one
// context, or the field-driven pairs) without type-1 coefficient grids, 1
// the large block (multi-context plans), 2 the small block compiled for
// type-10 operators only, 3 the small block with type-1 coefficient grids.
// The host code in sg4_device.cu reaches them through the entries defined
// here.
#include "sg4_items.cuh"

#ifndef EVR_GEO
#error "compile with -DEVR_GEO=0 (wide), 1 (narrow) or 2 (mid)"
#endif
#ifndef EVR_KIND
#error "compile with -DEVR_KIND=0 (small parameter block), 1 (large), 2 (small, type 10 only) or 3 (small, grids)"
#endif

namespace evr {

#if EVR_GEO == 0
#define EVR_G_CTAS EVR_WIDE_CTAS
#define EVR_G_FMAX EVR_WIDE_FMAX
#elif EVR_GEO == 1
#define EVR_G_CTAS EVR_NARROW_CTAS
#define EVR_G_FMAX EVR_NARROW_FMAX
#else
#define EVR_G_CTAS EVR_MID_CTAS
#define EVR_G_FMAX EVR_MID_FMAX
#endif

#define EVR_K_CAP (EVR_KIND == 1 ? EVR_PB_LARGE : EVR_PB_SMALL)
#define EVR_K_OPK (EVR_KIND == 2 ? 10 : (EVR_KIND == 0 ? 0 : 1))
#define EVR_K_KERNEL hpsi_items_kernel<EVR_G_CTAS, EVR_G_FMAX, EVR_K_CAP, EVR_K_OPK>

static void k_launch(unsigned grid, size_t smem, cudaStream_t s, const ParamBlock<EVR_K_CAP>& P, const MItem* items,
                     int n_items, int item_base, unsigned int* counter) {
  EVR_K_KERNEL<<<grid, EVR_CTA_THREADS, smem, s>>>(P, items, n_items, item_base, counter);
}

static cudaError_t k_static_smem(size_t* bytes) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, EVR_K_KERNEL);
  if (e == cudaSuccess) *bytes = a.sharedSizeBytes;
  return e;
}

static cudaError_t k_set_smem(int bytes) {
  return cudaFuncSetAttribute(EVR_K_KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

#if EVR_KIND == 0
#if EVR_GEO == 0
const MultiEntry<EVR_PB_SMALL> multi_small_wide = {k_launch, k_static_smem, k_set_smem};
#elif EVR_GEO == 1
const MultiEntry<EVR_PB_SMALL> multi_small_narrow = {k_launch, k_static_smem, k_set_smem};
#else
const MultiEntry<EVR_PB_SMALL> multi_small_mid = {k_launch, k_static_smem, k_set_smem};
#endif
#elif EVR_KIND == 1
#if EVR_GEO == 0
const MultiEntry<EVR_PB_LARGE> multi_large_wide = {k_launch, k_static_smem, k_set_smem};
#elif EVR_GEO == 1
const MultiEntry<EVR_PB_LARGE> multi_large_narrow = {k_launch, k_static_smem, k_set_smem};
#else
const MultiEntry<EVR_PB_LARGE> multi_large_mid = {k_launch, k_static_smem, k_set_smem};
#endif
#elif EVR_KIND == 2
#if EVR_GEO == 0
const MultiEntry<EVR_PB_SMALL> multi_small10_wide = {k_launch, k_static_smem, k_set_smem};
#elif EVR_GEO == 1
const MultiEntry<EVR_PB_SMALL> multi_small10_narrow = {k_launch, k_static_smem, k_set_smem};
#else
const MultiEntry<EVR_PB_SMALL> multi_small10_mid = {k_launch, k_static_smem, k_set_smem};
#endif
#else
#if EVR_GEO == 0
const MultiEntry<EVR_PB_SMALL> multi_small1g_wide = {k_launch, k_static_smem, k_set_smem};
#elif EVR_GEO == 1
const MultiEntry<EVR_PB_SMALL> multi_small1g_narrow = {k_launch, k_static_smem, k_set_smem};
#else
const MultiEntry<EVR_PB_SMALL> multi_small1g_mid = {k_launch, k_static_smem, k_set_smem};
#endif
#endif

}  // namespace evr
