// InputPort.h -- reference header name (ptask/InputPort.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_INPUTPORT_H
#define PTASK_GB300_FWD_INPUTPORT_H
#include "ptask_core.h"
#endif
