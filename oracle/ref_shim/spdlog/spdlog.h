// Stand-in for the un-vendored spdlog submodule (ext/spdlog): logging is a no-op.
#pragma once
namespace spdlog {
template <typename... A> void info(const A&...) {}
template <typename... A> void warn(const A&...) {}
template <typename... A> void error(const A&...) {}
template <typename... A> void critical(const A&...) {}
template <typename... A> void debug(const A&...) {}
}  // namespace spdlog
