// Minimal stand-in for the spdlog logging library, used only to compile the
// reference fast-bc headers and CLI in this container (spdlog is not installed).
// It holds no arithmetic: every logging macro discards its arguments, so the
// reference's numerical behaviour is unaffected.
#pragma once
#include <memory>
#include <string>

#define SPDLOG_LEVEL_TRACE 0
#define SPDLOG_LEVEL_DEBUG 1
#define SPDLOG_LEVEL_INFO 2
#define SPDLOG_LEVEL_WARN 3
#define SPDLOG_LEVEL_ERROR 4
#define SPDLOG_LEVEL_CRITICAL 5
#define SPDLOG_LEVEL_OFF 6
#ifndef SPDLOG_ACTIVE_LEVEL
#define SPDLOG_ACTIVE_LEVEL SPDLOG_LEVEL_INFO
#endif

#define SPDLOG_TRACE(...) ((void)0)
#define SPDLOG_DEBUG(...) ((void)0)
#define SPDLOG_INFO(...) ((void)0)
#define SPDLOG_WARN(...) ((void)0)
#define SPDLOG_ERROR(...) ((void)0)
#define SPDLOG_CRITICAL(...) ((void)0)

namespace spdlog {
struct logger {};
namespace level {
enum level_enum { trace = 0, debug, info, warn, err, critical, off };
inline level_enum from_str(const std::string& s) {
    if (s == "trace") return trace;
    if (s == "debug") return debug;
    if (s == "info") return info;
    if (s == "warning" || s == "warn") return warn;
    if (s == "error") return err;
    if (s == "critical") return critical;
    return off;
}
}  // namespace level
inline void set_default_logger(std::shared_ptr<logger>) {}
inline void set_pattern(const std::string&) {}
inline void set_level(level::level_enum) {}
}  // namespace spdlog
