// primitive_types.h -- basic types, enums and control signals of the PTask API
// (reference: ptask/primitive_types.h).  Values of every enum and signal match the reference so
// that code written against the reference keeps its meaning.  The Win32 scalar types the reference
// API uses (BOOL, UINT, DWORD, ...) are defined here for non-Windows hosts.
#ifndef PTASK_GB300_PRIMITIVE_TYPES_H
#define PTASK_GB300_PRIMITIVE_TYPES_H

#include <cmath>   // the reference's Win32 headers make fabs/sqrt visible to its sources
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#ifndef _WIN32
typedef int BOOL;
typedef unsigned int UINT;
typedef uint32_t DWORD;
typedef unsigned char BYTE;
typedef int64_t __int64;
typedef uint64_t UINT64;
typedef void *HANDLE;
typedef void VOID;
#ifndef TRUE
#define TRUE 1
#endif
#ifndef FALSE
#define FALSE 0
#endif
#ifndef INFINITE
#define INFINITE 0xFFFFFFFFu
#endif
#ifndef __stdcall
#define __stdcall
#endif
#ifndef sprintf_s
#define sprintf_s snprintf
#endif
#endif

namespace PTask {

// Result codes (ptask/primitive_types.h:33-77): > 0 failure, < 0 success with a warning.
typedef long PTRESULT;
const PTRESULT PTASK_OK = 0;
const PTRESULT PTASK_ERR = 1;
const PTRESULT PTASK_ERR_NOT_FOUND = 2;
const PTRESULT PTASK_ERR_INVALID_PARAMETER = 3;
const PTRESULT PTASK_ERR_EXISTS = 4;
const PTRESULT PTASK_ERR_GRAPH_MALFORMED = 4;
const PTRESULT PTASK_ERR_UNINITIALIZED = 5;
const PTRESULT PTASK_ERR_INFLIGHT = 6;
const PTRESULT PTASK_ERR_TOO_MANY_ACCELERATORS = 7;
const PTRESULT PTASK_ERR_ALREADY_INITIALIZED = 8;
const PTRESULT PTASK_WARNING = -1;
const PTRESULT PTASK_WARNING_GRAPH_MALFORMED = -2;
#define PTSUCCESS(x) ((x) <= PTask::PTASK_OK)
#define PTFAILED(x) ((x) > PTask::PTASK_OK)

typedef unsigned int PORTINDEX;

// Accelerator classes (only CUDA is backed by code here).
typedef enum acctype_t {
    ACCELERATOR_CLASS_DIRECT_X = 0,
    ACCELERATOR_CLASS_OPEN_CL = 1,
    ACCELERATOR_CLASS_CUDA = 2,
    ACCELERATOR_CLASS_REFERENCE = 3,
    ACCELERATOR_CLASS_HOST = 4,
    ACCELERATOR_CLASS_UNKNOWN = 5
} ACCELERATOR_CLASS;

typedef unsigned int BUFFERACCESSFLAGS;
const BUFFERACCESSFLAGS PT_ACCESS_DEFAULT = 0x0;
const BUFFERACCESSFLAGS PT_ACCESS_HOST_READ = 0x1;
const BUFFERACCESSFLAGS PT_ACCESS_HOST_WRITE = 0x2;
const BUFFERACCESSFLAGS PT_ACCESS_ACCELERATOR_READ = 0x4;
const BUFFERACCESSFLAGS PT_ACCESS_ACCELERATOR_WRITE = 0x8;
const BUFFERACCESSFLAGS PT_ACCESS_IMMUTABLE = 0x10;
const BUFFERACCESSFLAGS PT_ACCESS_BYTE_ADDRESSABLE = 0x20;

// Kernel parameter kinds (primitive_types.h:328-342).
typedef enum ptask_parm_t {
    PTPARM_INT = 0,
    PTPARM_FLOAT = 1,
    PTPARM_DOUBLE = 2,
    PTPARM_BYVALSTRUCT = 3,
    PTPARM_BYREFSTRUCT = 4,
    PTPARM_BUFFER = 5,
    PTPARM_NONE = 6
} PTASK_PARM_TYPE;

// Control signals carried by datablocks (primitive_types.h:374-400).
typedef uint64_t CONTROLSIGNAL;
const CONTROLSIGNAL DBCTLC_NONE = 0x0;
const CONTROLSIGNAL DBCTLC_BOF = 0x1;
const CONTROLSIGNAL DBCTLC_EOF = 0x2;
const CONTROLSIGNAL DBCTLC_BEGINITERATION = 0x4;
const CONTROLSIGNAL DBCTLC_ENDITERATION = 0x8;
const CONTROLSIGNAL DBCTLC_ERR = 0x10;
const CONTROLSIGNAL DBCTLC_DEVNULL = 0x20;
#define TESTSIGNAL(x, y) (((x) & (y)) != 0)
#define HASSIGNAL(x) ((x) != PTask::DBCTLC_NONE)
const char *ControlSignalString(CONTROLSIGNAL s);

// Port kinds (primitive_types.h:508-556).
typedef enum porttyp_t {
    INPUT_PORT,
    OUTPUT_PORT,
    STICKY_PORT,
    META_PORT,
    INITIALIZER_PORT
} PORTTYPE;

typedef enum descfun_t {
    DF_SIZE,
    DF_EOF,
    DF_BOF,
    DF_METADATA_SPLITTER,
    DF_CONTROL_CODE,
    DF_BLOCK_UID,
    DF_DATA_SOURCE,
    DF_METADATA_SOURCE,
    DF_TEMPLATE_SOURCE,
    DF_DATA_DIMENSIONS
} DESCRIPTORFUNC;

// Meta-port functions (primitive_types.h:639-650).
typedef enum metafun_t {
    MF_NONE = 0,
    MF_ALLOCATION_SIZE = 1,
    MF_SIMPLE_ITERATOR = 2,
    MF_GENERAL_ITERATOR = 3,
    MF_PADDED_ALLOCATION_SIZE = 4,
    MF_USER_DEFINED = 5
} METAFUNCTION;

typedef enum viewmaterializationpolicy_t {
    VIEWMATERIALIZATIONPOLICY_ON_DEMAND = 0,
    VIEWMATERIALIZATIONPOLICY_EAGER = 1
} VIEWMATERIALIZATIONPOLICY;
const char *ViewPolicyString(VIEWMATERIALIZATIONPOLICY p);

typedef struct ptask_dim3_t {
    int x, y, z;
    ptask_dim3_t(int xx = 1, int yy = 1, int zz = 1) : x(xx), y(yy), z(zz) {}
} PTASKDIM3;

typedef enum schedmode_t {
    SCHEDMODE_COOPERATIVE = 0,
    SCHEDMODE_PRIORITY = 1,
    SCHEDMODE_DATADRIVEN = 2,
    SCHEDMODE_FIFO = 3
} SCHEDULINGMODE;

typedef enum threadpoolpolicy_t {
    TPP_AUTOMATIC = 0,
    TPP_EXPLICIT = 1,
    TPP_THREADPERTASK = 2
} THREADPOOLPOLICY;

typedef enum _graph_state_t {
    PTGS_INITIALIZING = 0,
    PTGS_RUNNABLE = 1,
    PTGS_RUNNING = 2,
    PTGS_QUIESCING = 3,
    PTGS_TEARINGDOWN = 4,
    PTGS_TEARDOWNCOMPLETE = 5
} GRAPHSTATE;

// Channel predication (channel.h:33-196).
typedef enum chendpoint_t {
    CE_SRC = 0,
    CE_DST = 1
} CHANNELENDPOINTTYPE;

typedef enum chpred_t {
    CGATEFN_NONE = 0,
    CGATEFN_CLOSE_ON_EOF = 1,
    CGATEFN_OPEN_ON_EOF = 2,
    CGATEFN_OPEN_ON_BEGINITERATION = 3,
    CGATEFN_CLOSE_ON_BEGINITERATION = 4,
    CGATEFN_OPEN_ON_ENDITERATION = 5,
    CGATEFN_CLOSE_ON_ENDITERATION = 6,
    CGATEFN_DEVNULL = 7,
    CGATEFN_CLOSE_ON_BOF = 8,
    CGATEFN_OPEN_ON_BOF = 9,
    CGATEFN_USER_DEFINED = 10
} CHANNELPREDICATE;

typedef enum chtype_t {
    CT_GRAPH_INPUT = 0,
    CT_GRAPH_OUTPUT = 1,
    CT_INTERNAL = 2,
    CT_MULTI = 3,
    CT_INITIALIZER = 4
} CHANNELTYPE;

}  // namespace PTask

#endif
