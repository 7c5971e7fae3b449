// multichannel.h -- reference header name (ptask/multichannel.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_MULTICHANNEL_H
#define PTASK_GB300_FWD_MULTICHANNEL_H
#include "ptask_core.h"
#endif
