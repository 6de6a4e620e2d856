// Shim for the reference build only (oracle/_ref): the reference's Logger macros (include/util/Logger.h)
// writing to stderr.
#pragma once
#include <cstdio>
#include <string>
#define LOG_INFO(msg) {}
#define LOG_WARN(msg) {}
#define LOG_ERROR(msg) { std::fprintf(stderr, "[ref] %s\n", std::string(msg).c_str()); }
#define LOG_FATAL(msg) { std::fprintf(stderr, "[ref] %s\n", std::string(msg).c_str()); }
