// Compile-time simulator switches (same macro names and defaults as the
// reference include/SimConfigs.h:3-6).
#pragma once

// #define ENABLE_SIM_PROFILE   // per-partition clock64 profile in free-running mode

#define PROFILE_START_CYCLE 100
#define PROFILE_COLLECT_CYCLE 100
