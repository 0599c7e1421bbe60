// Generated by csrc/gen_cosx.py -- do not edit by hand.
// Packed primitive-pair record of each class (class order):
// float4 count = 2 (P hi, P lo) + n_om (omega record) + n_e (E).
#pragma once

namespace wb {
constexpr int kRecNom[10] = {1, 2, 2, 2, 3, 3, 3, 3, 4, 4};
constexpr int kRecNe[10] = {0, 2, 6, 4, 11, 20, 7, 18, 31, 48};
constexpr int kRecStride[10] = {3, 6, 10, 8, 16, 25, 12, 23, 37, 54};
}  // namespace wb
