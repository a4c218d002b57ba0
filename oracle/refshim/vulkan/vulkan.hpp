// Stand-in for the Vulkan-Hpp header, used only to compile reference sources
// for the test oracle: Span.h (the octree builder) needs vk::ArrayProxy, the
// headless.conf parser the 2D offset, extent and rectangle structs.
#pragma once
#include <cstddef>
#include <cstdint>
namespace vk {
template <typename T>
class ArrayProxy {
public:
    size_t size() const { return 0; }
    const T* data() const { return nullptr; }
};
struct Offset2D {
    int32_t x = 0, y = 0;
};
struct Extent2D {
    uint32_t width = 0, height = 0;
};
struct Rect2D {
    Offset2D offset;
    Extent2D extent;
};
}
