// accelerator.h -- reference header name (ptask/accelerator.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_ACCELERATOR_H
#define PTASK_GB300_FWD_ACCELERATOR_H
#include "ptask_core.h"
#endif
