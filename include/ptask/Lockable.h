// Lockable.h -- reference header name (ptask/Lockable.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_LOCKABLE_H
#define PTASK_GB300_FWD_LOCKABLE_H
#include "ptask_core.h"
#endif
