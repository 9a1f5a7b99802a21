/* count32_batch.cu -- instantiations of the FP32 counting kernel for a
 * batch of periodic boxes in one persistent launch. */
#include "count32.cuh"

kfun_t fcfcg_pick32_batch(int bin, int wt) {
#define K32(B)                                                             \
  if (bin == B)                                                            \
    return wt ? (kfun_t) k_count32<FCFCG_GEOM_BOX, B, 1, 1, 0>             \
              : (kfun_t) k_count32<FCFCG_GEOM_BOX, B, 0, 1, 0>;
  K32(FCFCG_BIN_ISO)
  K32(FCFCG_BIN_SMU)
  K32(FCFCG_BIN_SPI)
  K32(BIN_SPIL)
  K32(BIN_ISOL)
  K32(BIN_SMUL)
  K32(BIN_ISOLIN)
  K32(BIN_SMULIN)
#undef K32
  return 0;
}
