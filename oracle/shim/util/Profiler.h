// Shim for the reference build only (oracle/_ref): the reference's Profiler (include/util/Profiler.h)
// reduced to its call surface with no-op timers.
#pragma once
#include <string>
#define PROFILE(name, code) { profiler->start(name); code profiler->stop(name); }
#define PROFILE_FULL(name, code) { Profiler* profiler = Profiler::Get(); profiler->start(name); code profiler->stop(name); }
class Profiler {
public:
    static Profiler* Get() { static Profiler p; return &p; }
    void start(const std::string&) {}
    void stop(const std::string&) {}
};
