// Reference-CUDA build shim (test infrastructure only): type-checking stand-in
// for silver_bullets::sync::SyncAccessor (host code of the render unit).
#pragma once
#include <mutex>
namespace silver_bullets {
namespace sync {
template <class T, class M> class SyncAccessor {
public:
    T& access() { return m_value; }
    const T& access() const { return m_value; }
private:
    T m_value{};
    mutable M m_mutex;
};
} // namespace sync
} // namespace silver_bullets
