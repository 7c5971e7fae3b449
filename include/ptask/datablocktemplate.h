// datablocktemplate.h -- reference header name (ptask/datablocktemplate.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_DATABLOCKTEMPLATE_H
#define PTASK_GB300_FWD_DATABLOCKTEMPLATE_H
#include "ptask_core.h"
#endif
