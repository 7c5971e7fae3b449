// InitializerChannel.h -- reference header name (ptask/InitializerChannel.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_INITIALIZERCHANNEL_H
#define PTASK_GB300_FWD_INITIALIZERCHANNEL_H
#include "ptask_core.h"
#endif
