// gpusort/gpusort.h - all entry points of gpusort_gb300's C++ layer.
#ifndef GPUSORT_GB300_GPUSORT_H_
#define GPUSORT_GB300_GPUSORT_H_

#include "hyksort.h"
#include "hyperquicksort.h"
#include "samplesort.h"

#endif  // GPUSORT_GB300_GPUSORT_H_
