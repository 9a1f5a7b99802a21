/* count32_survey.cu -- instantiations of the FP32 counting kernel for
 * survey catalogues (no periodic images, midpoint line of sight). */
#include "count32.cuh"

kfun_t fcfcg_pick32_survey(int bin, int wt) {
#define K32(B)                                                             \
  if (bin == B)                                                            \
    return wt ? (kfun_t) k_count32<FCFCG_GEOM_SURVEY, B, 1, 0, 0>          \
              : (kfun_t) k_count32<FCFCG_GEOM_SURVEY, B, 0, 0, 0>;
  K32(FCFCG_BIN_ISO)
  K32(FCFCG_BIN_SMU)
  K32(FCFCG_BIN_SPI)
  K32(BIN_ISOLIN)
  K32(BIN_SMULIN)
#undef K32
  return 0;
}
