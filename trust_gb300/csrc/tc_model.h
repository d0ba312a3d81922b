// tc_model.h — layout of the per-vertex cost model (8 -> 32 -> 32 -> 1 MLP, fp32).
#pragma once

constexpr int TC_FEATURES = 8;
constexpr int TC_HIDDEN = 32;
constexpr int TC_OFF_MEAN = 0;                                      // feature means [8]
constexpr int TC_OFF_ISCALE = TC_OFF_MEAN + TC_FEATURES;            // 1 / feature std [8]
constexpr int TC_OFF_W1 = TC_OFF_ISCALE + TC_FEATURES;              // [32][8]
constexpr int TC_OFF_B1 = TC_OFF_W1 + TC_HIDDEN * TC_FEATURES;      // [32]
constexpr int TC_OFF_W2 = TC_OFF_B1 + TC_HIDDEN;                    // [32][32]
constexpr int TC_OFF_B2 = TC_OFF_W2 + TC_HIDDEN * TC_HIDDEN;        // [32]
constexpr int TC_OFF_W3 = TC_OFF_B2 + TC_HIDDEN;                    // [32]
constexpr int TC_OFF_B3 = TC_OFF_W3 + TC_HIDDEN;                    // [1]
constexpr int TC_OFF_YMEAN = TC_OFF_B3 + 1;                         // target mean
constexpr int TC_OFF_YSCALE = TC_OFF_YMEAN + 1;                     // target std
constexpr int TC_MODEL_FLOATS = TC_OFF_YSCALE + 1;                  // 1395
