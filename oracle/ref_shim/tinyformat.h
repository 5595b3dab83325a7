// Stand-in for the un-vendored tinyformat submodule (ext/tinyformat): the
// reference uses tfm::format only for toString() and exception messages, which
// the harness never prints, so the format string is returned unformatted.
#pragma once
#include <string>
namespace tfm {
template <typename... Args> std::string format(const char* fmt, const Args&...) { return std::string(fmt); }
template <typename... Args> std::string format(const std::string& fmt, const Args&...) { return fmt; }
}  // namespace tfm
