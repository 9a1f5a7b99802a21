/* count32_adj.cu -- instantiations of the FP32 counting kernel's adjoint
 * (gradients of weighted counts with respect to the weights). */
#include "count32.cuh"

kfun_t fcfcg_pick32_adj(int geom, int bin) {
#define K32A(G, B)                                                         \
  if (geom == G && bin == B) return (kfun_t) k_count32<G, B, 1, 0, 1>;
  K32A(FCFCG_GEOM_BOX, FCFCG_BIN_ISO)
  K32A(FCFCG_GEOM_BOX, FCFCG_BIN_SMU)
  K32A(FCFCG_GEOM_BOX, FCFCG_BIN_SPI)
  K32A(FCFCG_GEOM_SURVEY, FCFCG_BIN_ISO)
  K32A(FCFCG_GEOM_SURVEY, FCFCG_BIN_SMU)
  K32A(FCFCG_GEOM_SURVEY, FCFCG_BIN_SPI)
  K32A(FCFCG_GEOM_BOX, BIN_SPIL)
  K32A(FCFCG_GEOM_BOX, BIN_ISOL)
  K32A(FCFCG_GEOM_BOX, BIN_SMUL)
  K32A(FCFCG_GEOM_BOX, BIN_ISOLIN)
  K32A(FCFCG_GEOM_BOX, BIN_SMULIN)
  K32A(FCFCG_GEOM_SURVEY, BIN_ISOLIN)
  K32A(FCFCG_GEOM_SURVEY, BIN_SMULIN)
#undef K32A
  return 0;
}
