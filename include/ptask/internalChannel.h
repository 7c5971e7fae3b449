// internalChannel.h -- reference header name (ptask/internalChannel.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_INTERNALCHANNEL_H
#define PTASK_GB300_FWD_INTERNALCHANNEL_H
#include "ptask_core.h"
#endif
