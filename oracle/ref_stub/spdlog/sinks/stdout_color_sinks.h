// Stand-in for spdlog's colour console sink factory (see ../spdlog.h).
#pragma once
#include "../spdlog.h"
namespace spdlog {
inline std::shared_ptr<logger> stdout_color_mt(const std::string&) { return std::make_shared<logger>(); }
}  // namespace spdlog
