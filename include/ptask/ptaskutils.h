// ptaskutils.h -- small helpers of the reference's ptaskutils namespace (ptask/ptaskutils.h).
#ifndef PTASK_GB300_PTASKUTILS_H
#define PTASK_GB300_PTASKUTILS_H
#include "primitive_types.h"
namespace PTask {
namespace ptaskutils {
// Index of the lowest set bit of a control signal, -1 when none.
inline int GetFirstSignalIndex(CONTROLSIGNAL s)
{
    for (int i = 0; i < 64; ++i)
        if (s & (1ull << i)) return i;
    return -1;
}
inline UINT nextpowerof2(UINT v)
{
    UINT p = 1;
    while (p < v) p <<= 1;
    return p;
}
}  // namespace ptaskutils
}  // namespace PTask
#endif
