// channel.h -- reference header name (ptask/channel.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_CHANNEL_H
#define PTASK_GB300_FWD_CHANNEL_H
#include "ptask_core.h"
#endif
