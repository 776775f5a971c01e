#pragma once
// std::allocator over an Arena, or the heap when the arena is null; a refusal throws
// std::bad_alloc (raw/core/arena_allocator.hpp).
#include "raw/core/arena.hpp"
#include <cstddef>
#include <new>
#include <type_traits>
namespace raw {
template <class T>
struct ArenaAllocator {
    using value_type = T;
    using propagate_on_container_copy_assignment = std::true_type;
    using propagate_on_container_move_assignment = std::true_type;
    using propagate_on_container_swap = std::true_type;
    using is_always_equal = std::false_type;
    Arena* arena_{nullptr};
    ArenaAllocator() noexcept = default;
    explicit ArenaAllocator(Arena* a) noexcept : arena_(a) {}
    template <class U> ArenaAllocator(const ArenaAllocator<U>& o) noexcept : arena_(o.arena_) {}
    T* allocate(std::size_t n) {
        void* p = arena_ ? arena_->allocate(n * sizeof(T), alignof(T)) : ::operator new(n * sizeof(T));
        if (!p) throw std::bad_alloc();
        return static_cast<T*>(p);
    }
    void deallocate(T* p, std::size_t) noexcept { if (!arena_) ::operator delete(p); }
    template <class U> bool operator==(const ArenaAllocator<U>& o) const noexcept { return arena_ == o.arena_; }
    template <class U> bool operator!=(const ArenaAllocator<U>& o) const noexcept { return arena_ != o.arena_; }
};
}  // namespace raw
