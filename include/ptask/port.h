// port.h -- reference header name (ptask/port.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_PORT_H
#define PTASK_GB300_FWD_PORT_H
#include "ptask_core.h"
#endif
