// graphOutputChannel.h -- reference header name (ptask/graphOutputChannel.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_GRAPHOUTPUTCHANNEL_H
#define PTASK_GB300_FWD_GRAPHOUTPUTCHANNEL_H
#include "ptask_core.h"
#endif
