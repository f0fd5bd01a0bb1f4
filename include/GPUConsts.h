// Kept for source compatibility with include/GPUConsts.h:3 of the reference
// (the constant is unused there as well).
#pragma once

#define GPUMemPaddingSize 128
