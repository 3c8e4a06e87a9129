// CL/cl2.hpp -- the few OpenCL C++ declarations that the engine's OpenCL.h
// and Network.cpp name, for building the engine's OpenCL configuration
// (config.h: USE_OPENCL) on the GB300 path without an OpenCL SDK.
//
// Nothing here talks to an OpenCL device: the classes only hold what the
// engine's weight-upload templates (OpenCL.h:66-87) hand over, and
// opencl_gb300.cpp -- which replaces the engine's OpenCL.cpp -- reads the
// weights back from them and runs the nets through leela_gpu.h.
#ifndef LEELA_GB300_FAKE_CL2_HPP
#define LEELA_GB300_FAKE_CL2_HPP

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

typedef int32_t cl_int;
typedef uint64_t cl_mem_flags;
typedef struct _cl_event *cl_event;

#ifndef CL_CALLBACK
#define CL_CALLBACK
#endif
#define CL_COMPLETE 0x0
#define CL_SUCCESS 0
#define CL_MEM_READ_WRITE (1 << 0)
#define CL_MEM_WRITE_ONLY (1 << 1)
#define CL_MEM_READ_ONLY (1 << 2)
#define CL_MEM_COPY_HOST_PTR (1 << 5)
#define CL_MEM_HOST_NO_ACCESS (1 << 9)

namespace cl {

// A host copy of what was handed over (CL_MEM_COPY_HOST_PTR), shared by the
// copies of the object the engine's containers make.
class Buffer {
public:
    Buffer() = default;
    Buffer(cl_mem_flags, size_t bytes, void *host = nullptr)
        : m_data(std::make_shared<std::vector<unsigned char>>(bytes)) {
        if (host && bytes) std::memcpy(m_data->data(), host, bytes);
    }
    size_t size() const { return m_data ? m_data->size() : 0; }
    const float *floats() const { return m_data ? reinterpret_cast<const float *>(m_data->data()) : nullptr; }

private:
    std::shared_ptr<std::vector<unsigned char>> m_data;
};

class CommandQueue {};
class Kernel {};
class Program {};

}  // namespace cl

#endif
