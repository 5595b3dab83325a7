// Stand-in for the un-vendored wjakob/filesystem submodule (file resolver).
#pragma once
#include "filesystem/path.h"
namespace filesystem {
class resolver {
public:
    path resolve(const path& p) const { return p; }
    void prepend(const path&) {}
    void append(const path&) {}
};
}  // namespace filesystem
