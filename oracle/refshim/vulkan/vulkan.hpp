// Stand-in for the Vulkan-Hpp header, used only to compile the reference's
// octree builder (test oracle). Span.h needs nothing but vk::ArrayProxy.
#pragma once
#include <cstddef>
namespace vk {
template <typename T>
class ArrayProxy {
public:
    size_t size() const { return 0; }
    const T* data() const { return nullptr; }
};
}
