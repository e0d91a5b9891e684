// Stand-in for the reference's spdlog-based logger (Backend/includes/tools/logger/logger.hh) when
// its hot-path translation units are compiled as the comparison build: every LOG_* macro is a no-op
// and CHECK reports to stderr and aborts, so no logging library is needed.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <exception>
#include <memory>
#include <string>

#define LOG_TRACE(...) ((void)0)
#define LOG_DEBUG(...) ((void)0)
#define LOG_INFO(...) ((void)0)
#define LOG_WARN(...) ((void)0)
#define LOG_ERROR(...) ((void)0)
#define LOG_CRITICAL(...) ((void)0)
#define LOG_FUNC(...) ((void)0)
#define CODE_WITH_NO_LOG(statement) \
    {                               \
        statement;                  \
    }
#define CUDA_FATAL(file, line, fmt, ...)                                  \
    {                                                                     \
        std::fprintf(stderr, "comparison build: CUDA error at %s:%d\n", file, line); \
        std::abort();                                                     \
    }

#ifndef CHECK
#define HVREF_CHECK_FIRST(cond, ...) (cond)
#define CHECK(...)                                                                             \
    do                                                                                         \
    {                                                                                          \
        if (!(HVREF_CHECK_FIRST(__VA_ARGS__, 0)))                                              \
        {                                                                                      \
            std::fprintf(stderr, "comparison build: CHECK failed at %s:%d\n", __FILE__, __LINE__); \
            std::abort();                                                                      \
        }                                                                                      \
    } while (0)
#endif
