// Stand-in for Velvet/VtBuffer.hpp when the reference's solver sources are compiled on the
// CPU — TEST INFRASTRUCTURE.  Velvet/SpatialHashGPU.cu keeps its sort scratch in a
// VtBuffer<void*> and passes it as the scratch pointer; this growable host buffer is all
// it needs (the real file's OpenGL-interop buffers are not used by the solver kernels).
#pragma once

#include <cstdlib>

#include "Common.cuh"

namespace Velvet {

template <class T>
class VtBuffer {
public:
    VtBuffer() {}
    VtBuffer(const VtBuffer&) = delete;
    VtBuffer& operator=(const VtBuffer&) = delete;
    ~VtBuffer() { std::free(m_buffer); }
    operator T*() const { return m_buffer; }
    size_t size() const { return m_count; }
    void resize(size_t n)
    {
        T* p = static_cast<T*>(std::realloc(m_buffer, (n ? n : 1) * sizeof(T)));
        if (!p) std::abort();
        m_buffer = p;
        m_count = n;
    }

private:
    T* m_buffer = nullptr;
    size_t m_count = 0;
};

}  // namespace Velvet
