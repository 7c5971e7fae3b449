// ptaskapi.h -- public API of the GB300 PTask runtime (reference: ptask/ptaskapi.h:11-31).
#ifndef PTASK_GB300_PTASKAPI_H
#define PTASK_GB300_PTASKAPI_H
#include "primitive_types.h"
#include "PTaskRuntime.h"
#include "ptaskutils.h"
#include "accelerator.h"
#include "graph.h"
#include "datablock.h"
#include "datablocktemplate.h"
#include "CompiledKernel.h"
#include "hrperft.h"
#include "task.h"
#include "graphInputChannel.h"
#include "graphOutputChannel.h"
#include "internalChannel.h"
#include "InitializerChannel.h"
#include "multichannel.h"
#include "InputPort.h"
#include "OutputPort.h"
#include "StickyPort.h"
#include "MetaPort.h"
#include "shrperft.h"
#endif
