// OutputPort.h -- reference header name (ptask/OutputPort.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_OUTPUTPORT_H
#define PTASK_GB300_FWD_OUTPUTPORT_H
#include "ptask_core.h"
#endif
