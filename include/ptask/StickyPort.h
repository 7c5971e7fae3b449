// StickyPort.h -- reference header name (ptask/StickyPort.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_STICKYPORT_H
#define PTASK_GB300_FWD_STICKYPORT_H
#include "ptask_core.h"
#endif
