// Generated by csrc/gen_cosx.py -- do not edit by hand.
// Packed primitive-pair record of each class (class order):
// float4 count = 2 (P hi, P lo) + n_om (omega record) + n_e (E).
#pragma once

namespace wb {
constexpr int kRecNom[10] = {2, 3, 3, 3, 4, 4, 4, 4, 5, 5};
constexpr int kRecNe[10] = {0, 2, 6, 4, 11, 20, 7, 18, 31, 48};
constexpr int kRecStride[10] = {4, 7, 11, 9, 17, 26, 13, 24, 38, 55};
// dual-omega record: 2 + 2 n_om + n_e
constexpr int kRecStride2[10] = {6, 10, 14, 12, 21, 30, 17, 28, 43, 60};
}  // namespace wb
