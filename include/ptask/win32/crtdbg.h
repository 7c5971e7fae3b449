/* crtdbg.h -- the MSVC debug-heap header has no counterpart off Windows; the macros the reference's
 * test code uses become no-ops. */
#ifndef PTASK_GB300_CRTDBG_H
#define PTASK_GB300_CRTDBG_H
#define _CrtSetDbgFlag(x) (0)
#define _CrtDumpMemoryLeaks() (0)
#define _CRTDBG_ALLOC_MEM_DF 0
#define _CRTDBG_LEAK_CHECK_DF 0
#endif
