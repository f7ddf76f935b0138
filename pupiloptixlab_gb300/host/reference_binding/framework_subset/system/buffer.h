// Declaration subset of framework/system/buffer.h:13-63 without DX12: buffer
// flags and descriptor, Buffer (CUDA device pointer) and the named-buffer
// manager.  Outside the tree the manager allocates with cudaMalloc.
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <string_view>
#include <vector>
#include <cuda_runtime.h>
#include "util/util.h"

namespace Pupil {
using CUdeviceptr_t = unsigned long long;  // CUdeviceptr

enum class EBufferFlag : unsigned int { None = 0, SharedWithDX12 = 1, AllowDisplay = 1 << 1 };

struct BufferDesc {
    const char *name = nullptr;
    EBufferFlag flag = EBufferFlag::None;
    uint32_t width = 1;
    uint32_t height = 1;
    uint32_t stride_in_byte = 1;
};
struct Buffer {
    BufferDesc desc{};
    CUdeviceptr_t cuda_ptr = 0;
    Buffer() noexcept = default;
    Buffer(const BufferDesc &d) noexcept : desc(d) {}
    ~Buffer() noexcept { if (cuda_ptr) cudaFree(reinterpret_cast<void *>(cuda_ptr)); }
};
class BufferManager : public util::Singleton<BufferManager> {
public:
    constexpr static std::string_view DEFAULT_FINAL_RESULT_BUFFER_NAME = "final result";
    Buffer *GetBuffer(std::string_view id) noexcept {
        auto it = m_buffers.find(std::string(id));
        return it == m_buffers.end() ? nullptr : it->second.get();
    }
    Buffer *AllocBuffer(const BufferDesc &desc) noexcept {
        auto b = std::make_unique<Buffer>(desc);
        const size_t bytes = (size_t)desc.width * desc.height * desc.stride_in_byte;
        void *p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        b->cuda_ptr = reinterpret_cast<CUdeviceptr_t>(p);
        Buffer *raw = b.get();
        m_names.push_back(desc.name);
        m_buffers[desc.name] = std::move(b);
        return raw;
    }
    const std::vector<std::string> &GetBufferNameList() const noexcept { return m_names; }

private:
    std::map<std::string, std::unique_ptr<Buffer>> m_buffers;
    std::vector<std::string> m_names;
};
}  // namespace Pupil
