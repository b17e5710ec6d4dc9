// mlp.h -- layout of the learned step proposer's parameters (mlp.cu).
#pragma once

namespace redgb {

constexpr int MLP_IN = 8;
constexpr int MLP_HIDDEN = 64;
constexpr int MLP_TB = 32;  // samples per CTA in the training kernels
constexpr int MLP_OFF_W1 = 0;
constexpr int MLP_OFF_B1 = MLP_OFF_W1 + MLP_HIDDEN * MLP_IN;
constexpr int MLP_OFF_W2 = MLP_OFF_B1 + MLP_HIDDEN;
constexpr int MLP_OFF_B2 = MLP_OFF_W2 + MLP_HIDDEN * MLP_HIDDEN;
constexpr int MLP_OFF_W3 = MLP_OFF_B2 + MLP_HIDDEN;
constexpr int MLP_OFF_B3 = MLP_OFF_W3 + MLP_HIDDEN;
constexpr int MLP_NPARAM = MLP_OFF_B3 + 1;

}  // namespace redgb
