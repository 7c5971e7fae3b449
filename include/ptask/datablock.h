// datablock.h -- reference header name (ptask/datablock.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_DATABLOCK_H
#define PTASK_GB300_FWD_DATABLOCK_H
#include "ptask_core.h"
#endif
