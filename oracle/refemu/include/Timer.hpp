// Stand-in for Velvet/Timer.hpp when the reference's solver sources are compiled on the
// CPU — TEST INFRASTRUCTURE.  The real file times frames with GLFW and CUDA events; the
// solver sources only construct ScopedTimerGPU around their launches, which times
// nothing here.
#pragma once

#include <string>

namespace Velvet {

class ScopedTimerGPU {
public:
    explicit ScopedTimerGPU(const std::string&&) {}
};

}  // namespace Velvet
