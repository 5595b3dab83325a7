// Stand-in for the un-vendored wjakob/filesystem submodule: only the type names
// are needed by include/core/base/common.h.
#pragma once
#include <string>
namespace filesystem {
class path {
public:
    path() {}
    path(const std::string& s) : s_(s) {}
    std::string str() const { return s_; }
private:
    std::string s_;
};
}  // namespace filesystem
