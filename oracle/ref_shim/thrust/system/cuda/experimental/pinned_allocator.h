// Stand-in for the pinned_allocator that older Thrust releases shipped: a
// plain std::allocator is enough for the host-side code compiled here.
#pragma once
#include <memory>
namespace thrust { namespace system { namespace cuda { namespace experimental {
template <typename T>
using pinned_allocator = std::allocator<T>;
}}}}
