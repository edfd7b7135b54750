// Host builders for the pair kernel's constant tables (see nddo_tables.cpp).
#pragma once
#include "nddo_math.cuh"

namespace nddo {
void build_eri_table(EriTable* t);
void build_overlap_table(OverlapTable* t);
}  // namespace nddo
