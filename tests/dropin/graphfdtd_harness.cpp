// Link harness for the reference's ptaskUnitTest/graphfdtd.cpp compiled, unmodified, against this
// runtime's include/ptask headers.  It supplies what the reference's test driver provides around
// that file (the globals of main.cpp and the helpers of platformcheck.cpp) and a main() that runs
// run_graph_fdtd_task the way main.cpp:1013-1015 does for `-t cufdtd`.
#include <cstdio>
#include <cstdlib>

#include "ptaskapi.h"
#include "graphfdtd.h"

BOOL g_bSingleThreaded = FALSE;
BOOL g_bEmulateModular = FALSE;
int g_nChannelCapacity = 4;
BOOL g_bSetChannelCapacity = FALSE;
BOOL g_verbose = FALSE;
char g_szCompilerOutputBuffer[4906];

int CheckPlatformSupport(char *szFile, char *)
{
    if (!PTask::Runtime::CanExecuteKernel(szFile)) {
        printf("platform cannot execute %s\n", szFile);
        exit(0);
    }
    return 1;
}

int CheckCompileSuccess(char *szfile, char *szshader, void *pKernel)
{
    if (!pKernel) {
        printf("%s:%s: compile failed: %s\n", szfile, szshader, g_szCompilerOutputBuffer);
        exit(1);
    }
    return 1;
}

// usage: graphfdtd_ref [rows cols depth blocks iterations]   (regtest.sh:1114 uses 64 64 4 4 4)
int main(int argc, char **argv)
{
    int r = argc > 1 ? atoi(argv[1]) : 64, c = argc > 2 ? atoi(argv[2]) : 64, z = argc > 3 ? atoi(argv[3]) : 4;
    int n = argc > 4 ? atoi(argv[4]) : 4, i = argc > 5 ? atoi(argv[5]) : 4;
    return run_graph_fdtd_task((char *)"fdtdKernels", (char *)"", r, c, z, n, i, CUDA);
}
