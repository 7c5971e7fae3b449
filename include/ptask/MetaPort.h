// MetaPort.h -- reference header name (ptask/MetaPort.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_METAPORT_H
#define PTASK_GB300_FWD_METAPORT_H
#include "ptask_core.h"
#endif
