// Test infrastructure (oracle build only): a std::chrono implementation of the
// reference's Timer interface (src/core/timer.h:3-19).  The reference's own
// src/core/timer.cpp uses QueryPerformanceCounter and <Windows.h>, so it cannot be
// compiled on Linux; this file stands in for it when the reference is built here.
#include <chrono>
#include "timer.h"

namespace {
using Clock = std::chrono::steady_clock;
}

Timer::Timer(void) : m_ctx(new Clock::time_point(Clock::now())) {}

float Timer::getTime(void)
{
    auto* start = static_cast<Clock::time_point*>(m_ctx);
    return std::chrono::duration<float>(Clock::now() - *start).count();
}

void Timer::reset(void)
{
    *static_cast<Clock::time_point*>(m_ctx) = Clock::now();
}

Timer::~Timer()
{
    delete static_cast<Clock::time_point*>(m_ctx);
}
