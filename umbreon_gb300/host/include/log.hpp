// Diagnostic routing of the umbreon API: a process-wide sink, stderr default.
#pragma once

#include <functional>

namespace umbreon {

enum class LogLevel { Warning, Info };
using LogSink = std::function<void(LogLevel level, const char* text)>;

void setLogSink(LogSink sink);
void logMessage(LogLevel level, const char* fmt, ...)
#if defined(__GNUC__) || defined(__clang__)
    __attribute__((format(printf, 2, 3)))
#endif
    ;

}  // namespace umbreon
