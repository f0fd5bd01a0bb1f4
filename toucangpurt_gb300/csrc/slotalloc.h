// Value-pool slot allocation (see slotalloc.cpp).
#pragma once
#include <cstdint>
#include <vector>

#include "ToucanGPUGenDataTypes.h"

namespace tgs {

constexpr uint32_t kNoSlot = 0xFFFFFFFFu;

// New number of every slot of the partition (kNoSlot: never accessed);
// returns the new pool size.
// keep (optional): slots that must hold their value until the partition ends
// (signal probes read them after the exec levels).
uint32_t planSlots(const toucanGPUSim::SimPartitionInfo &p, std::vector<uint32_t> &newOf,
                   const std::vector<uint32_t> *keep = nullptr);
// Rewrites every slot reference of the partition through newOf.
void renameSlots(toucanGPUSim::SimPartitionInfo &p, const std::vector<uint32_t> &newOf, uint32_t newSize);

}  // namespace tgs
