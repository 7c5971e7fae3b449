// graphInputChannel.h -- reference header name (ptask/graphInputChannel.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_GRAPHINPUTCHANNEL_H
#define PTASK_GB300_FWD_GRAPHINPUTCHANNEL_H
#include "ptask_core.h"
#endif
