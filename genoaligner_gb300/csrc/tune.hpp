// tune.hpp -- the per-device kernel settings the engine reads (tune.cu).
#pragma once

#include "../../include/genoaligner_gb300.h"

namespace ga {

// The setting for the calling thread's current device: the autotuner's
// candidate while it times one, else the device's stored setting, else the
// built-in default.  Read once per call, so one call uses one setting.
ga_tune tune_current();

}  // namespace ga
