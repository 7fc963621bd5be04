// Progress and warning messages of the host driver (the reference's Log, src/lib/Log.hpp):
// levels Debug < Info < Warning < Error, printed to stdout with a timestamp when at or
// above the display level.
#pragma once
#include <string>

namespace spn {

enum class LogLevel : int { Debug = 0, Info = 1, Warning = 2, Error = 3 };

void set_log_level(LogLevel display);
void log(LogLevel level, const std::string &msg);

}  // namespace spn
