// Stand-in for the x86 spin-wait hint utils/timer.hpp calls; a no-op keeps the
// harness portable (it only changes how a busy wait spins).
#pragma once
static inline void _mm_pause(void) {}
