// graph.h -- reference header name (ptask/graph.h); the declarations live in ptask_core.h.
#ifndef PTASK_GB300_FWD_GRAPH_H
#define PTASK_GB300_FWD_GRAPH_H
#include "ptask_core.h"
#endif
