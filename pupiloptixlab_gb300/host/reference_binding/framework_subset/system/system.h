// Declaration subset of framework/system/system.h:13-20: the system events.
#pragma once

namespace Pupil {
enum class ESystemEvent { Quit, Precompute, StartRendering, StopRendering, SceneLoad, FrameFinished };
}  // namespace Pupil
