// hrperft.h -- CHighResolutionTimer (reference: ptask/hrperft.h:33), on std::chrono.
#ifndef PTASK_GB300_HRPERFT_H
#define PTASK_GB300_HRPERFT_H
#include <chrono>

typedef enum hpfgran_t { gran_nanosec = 0, gran_usec = 1, gran_msec = 2, gran_sec = 3 } HPFGRANULARITY;

class CHighResolutionTimer {
public:
    explicit CHighResolutionTimer(HPFGRANULARITY g = gran_msec) : m_gran(g) { reset(); }
    void reset() { m_start = std::chrono::steady_clock::now(); m_last = m_start; }
    // Time since reset (or since the previous call when bReset) in the timer's granularity.
    double elapsed(bool bReset = false)
    {
        auto now = std::chrono::steady_clock::now();
        double s = std::chrono::duration<double>(now - (bReset ? m_last : m_start)).count();
        if (bReset) m_last = now;
        switch (m_gran) {
        case gran_nanosec: return s * 1e9;
        case gran_usec: return s * 1e6;
        case gran_msec: return s * 1e3;
        default: return s;
        }
    }
    double lap() { return elapsed(true); }

private:
    HPFGRANULARITY m_gran;
    std::chrono::steady_clock::time_point m_start, m_last;
};
#endif
