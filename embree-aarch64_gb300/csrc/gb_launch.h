// gb_launch.h -- process-wide count of the kernels this library launches
// (reported through rtcgbGetKernelLaunchCount).
#pragma once

namespace gb {
void note_launches(unsigned n);
}  // namespace gb
