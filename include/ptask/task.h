// task.h -- reference header name (ptask/task.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_TASK_H
#define PTASK_GB300_FWD_TASK_H
#include "ptask_core.h"
#endif
