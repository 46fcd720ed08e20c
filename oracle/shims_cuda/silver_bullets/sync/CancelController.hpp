// Build shim (test infrastructure only): silver_bullets::sync::CancelController, as far as the reference's
// worker interface uses it -- a controller whose Checker tells whether a cancel was requested.
#pragma once
#include <atomic>
namespace silver_bullets {
namespace sync {
class CancelController {
public:
    class Checker {
    public:
        explicit Checker(const std::atomic<bool>& flag) : m_flag(flag) {}
        explicit operator bool() const { return m_flag.load(); }

    protected:
        const std::atomic<bool>& cancelled() const { return m_flag; }

    private:
        const std::atomic<bool>& m_flag;
    };
    Checker checker() const { return Checker(m_cancelled); }
    void cancel() { m_cancelled = true; }
    void resume() { m_cancelled = false; }

private:
    std::atomic<bool> m_cancelled{false};
};
} // namespace sync
} // namespace silver_bullets
