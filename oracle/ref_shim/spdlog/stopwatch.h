// ORACLE (test infrastructure only): the stopwatch lives in spdlog.h of this
// project-owned spdlog subset.
#include "spdlog.h"
