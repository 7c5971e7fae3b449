// PTaskRuntime.h -- PTask::Runtime, the global entry points of the API (reference:
// ptask/PTaskRuntime.h).  Same names, parameters and defaults as the reference for the calls an
// FDTD graph makes; string parameters are const-qualified so string literals bind without casts.
#ifndef PTASK_GB300_RUNTIME_H
#define PTASK_GB300_RUNTIME_H

#include <string>

#include "ptask_core.h"

namespace PTask {
namespace Runtime {

// Lifetime (PTaskRuntime.h:182, :214).
PTRESULT Initialize();
PTRESULT Terminate();
BOOL IsInitialized();

// Templates (PTaskRuntime.h:2142, :2213).
DatablockTemplate *GetDatablockTemplate(const char *lpszType, unsigned int uiStride, unsigned int x,
                                        unsigned int y, unsigned int z, bool bRecordStream = false,
                                        bool bRaw = false);
DatablockTemplate *GetDatablockTemplate(const char *lpszType, unsigned int uiStride, PTASK_PARM_TYPE pttype);
DatablockTemplate *GetDatablockTemplate(const char *lpszType);

// Ports (PTaskRuntime.h:675).  nKernelParameterIndex / nInOutParmOutputIndex of (UINT)-1 mean
// "not bound to a formal parameter" / "not an in-out parameter", as in the reference.
Port *CreatePort(PORTTYPE type, DatablockTemplate *pTemplate, UINT uiId, const char *lpszVariableBinding = nullptr,
                 UINT nKernelParameterIndex = (UINT)-1, UINT nInOutParmOutputIndex = (UINT)-1);

// Datablocks (PTaskRuntime.h:2253).  The caller holds one reference to the returned block.
Datablock *AllocateDatablock(DatablockTemplate *pTemplate, void *pInitData, UINT cbInitData, Channel *pDestChannel,
                             BUFFERACCESSFLAGS flags = 0, CONTROLSIGNAL uiBlockControlCode = 0);
Datablock *AllocateDatablock(DatablockTemplate *pTemplate, void *pInitData, UINT cbInitData,
                             BUFFERACCESSFLAGS flags, CONTROLSIGNAL uiBlockControlCode);

// Kernels (PTaskRuntime.h:540, :264).  The file name is recorded but not compiled: the entry is
// resolved to a linked sm_103a kernel of libptask_gb300.so.
CompiledKernel *GetCompiledKernel(const char *lpszFile, const char *lpszOperation,
                                  char *lpszCompilerOutput = nullptr, int uiCompilerOutput = 0,
                                  int tgx = 1, int tgy = 1, int tgz = 1);
BOOL CanExecuteKernel(const char *szAcceleratorCodeFileName);

// Configuration (PTaskRuntime.h:702-1970).  Only CUDA is backed by an implementation; selecting
// another backend is recorded and reported by CanExecuteKernel.
void SetUseCUDA(BOOL b);
BOOL GetUseCUDA();
void SetUseOpenCL(BOOL b);
BOOL GetUseOpenCL();
void SetUseDirectX(BOOL b);
BOOL GetUseDirectX();
void SetUseHost(BOOL b);
BOOL GetUseHost();
void SetVerbose(BOOL b);
BOOL GetVerbose();
void SetDefaultChannelCapacity(int n);
int GetDefaultChannelCapacity();
void SetSchedulingMode(SCHEDULINGMODE m);
SCHEDULINGMODE GetSchedulingMode();
void SetThreadPoolPolicy(THREADPOOLPOLICY p);
THREADPOOLPOLICY GetThreadPoolPolicy();
void SetMaximumConcurrency(int n);
int GetMaximumConcurrency();
void SetExitOnRuntimeFailure(BOOL bExit);
BOOL GetExitOnRuntimeFailure();
void SetDispatchWatchdogThreshold(DWORD ms);
DWORD GetDispatchWatchdogThreshold();

// Messages and errors (PTaskRuntime.h:1981-2040, :2376).  HandleError prints the message and, when
// ExitOnRuntimeFailure is set (default TRUE, as in the reference), exits the process.
BOOL HandleError(const char *szMessage, ...);
BOOL HandleError(const std::string &strError);
BOOL MandatoryInform(const char *szMessage, ...);
void Inform(const char *szMessage, ...);
void Inform(const std::string &s);
void Warning(const char *szMessage, UINT nLogLevel = 0xFFFFFFFF);
void Warning(const std::string &s, UINT nLogLevel = 0xFFFFFFFF);
void ErrorMessage(const char *szMessage, UINT nLogLevel = 0xFFFFFFFF);
void ErrorMessage(const std::string &s, UINT nLogLevel = 0xFFFFFFFF);
void Trace(const char *szMessage, ...);

// The accelerator this runtime drives.
Accelerator *GetAccelerator();

}  // namespace Runtime
}  // namespace PTask

#endif
