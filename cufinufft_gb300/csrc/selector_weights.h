// selector_weights.h -- trained parameters of the learned layout selector.
// Written by cufinufft_gb300/selector/train.py; kSelectorTrained = 0 means no
// trained network is compiled in and gpu_method 0 keeps the built-in rule.
#pragma once

namespace cfg {
constexpr int kSelectorTrained = 0;
constexpr float kSelMean[14] = {0};
constexpr float kSelStd[14] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
constexpr float kSelParams[1833] = {0};
}  // namespace cfg
