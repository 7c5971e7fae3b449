// shrperft.h -- reference header name (ptask/shrperft.h); the shared timer is CHighResolutionTimer.
#ifndef PTASK_GB300_SHRPERFT_H
#define PTASK_GB300_SHRPERFT_H
#include "hrperft.h"
#endif
