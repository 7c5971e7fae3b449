// CompiledKernel.h -- reference header name (ptask/CompiledKernel.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_COMPILEDKERNEL_H
#define PTASK_GB300_FWD_COMPILEDKERNEL_H
#include "ptask_core.h"
#endif
