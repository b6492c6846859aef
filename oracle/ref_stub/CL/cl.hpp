// Minimal stand-in for the OpenCL C++ bindings header, used ONLY to compile the
// reference's CPU code path (src/skewEngine.cuh, src/kernel*.h) into the test
// oracle under oracle/_ref.  The reference includes <CL/cl.hpp> unconditionally
// (skewEngine.cuh:21-24) but its CPU path never calls into OpenCL, so every
// member here is a no-op.  This is test infrastructure, not product code.
#ifndef SKE_ORACLE_CL_STUB_HPP
#define SKE_ORACLE_CL_STUB_HPP

#include <cstddef>
#include <string>
#include <utility>
#include <vector>

typedef int cl_int;
#define CL_SUCCESS 0
#define CL_TRUE 1
#define CL_FALSE 0
#define CL_MEM_READ_ONLY 1
#define CL_MEM_WRITE_ONLY 2
#define CL_MEM_READ_WRITE 4
#define CL_DEVICE_TYPE_GPU 4
#define CL_PROGRAM_BUILD_LOG 0x1183

namespace cl {

struct Device {};
struct Platform {
    static cl_int get(std::vector<Platform>*) { return 0; }
    cl_int getDevices(int, std::vector<Device>*) const { return 0; }
};
struct Context {
    Context() {}
    explicit Context(const Device&) {}
};
struct NDRange {
    NDRange() {}
    NDRange(size_t) {}
    NDRange(size_t, size_t) {}
    NDRange(size_t, size_t, size_t) {}
};
static const NDRange NullRange;
struct Buffer {
    Buffer() {}
    Buffer(const Context&, int, size_t) {}
};
struct Program {
    typedef std::vector<std::pair<const char*, size_t> > Sources;
    Program() {}
    Program(const Context&, const Sources&) {}
    cl_int build(const std::vector<Device>&) const { return 0; }
    template <int N> std::string getBuildInfo(const Device&) const { return std::string(); }
};
struct Kernel {
    Kernel() {}
    Kernel(const Program&, const char*) {}
    template <typename T> cl_int setArg(unsigned, const T&) { return 0; }
};
struct CommandQueue {
    CommandQueue() {}
    CommandQueue(const Context&, const Device&) {}
    template <typename T>
    cl_int enqueueFillBuffer(const Buffer&, T, size_t, size_t) { return 0; }
    cl_int enqueueWriteBuffer(const Buffer&, int, size_t, size_t, const void*) { return 0; }
    cl_int enqueueReadBuffer(const Buffer&, int, size_t, size_t, void*) { return 0; }
    cl_int enqueueNDRangeKernel(const Kernel&, const NDRange&, const NDRange&, const NDRange&) { return 0; }
    cl_int finish() { return 0; }
};

}  // namespace cl

#endif
