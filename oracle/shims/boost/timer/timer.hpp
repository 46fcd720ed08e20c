// Oracle build shim: boost::timer::cpu_timer on std::chrono (wall time only).
#pragma once
#include <chrono>
#include <cstdint>
#include <string>
namespace boost {
namespace timer {
using nanosecond_type = std::int64_t;
struct cpu_times {
    nanosecond_type wall = 0, user = 0, system = 0;
    void clear() { wall = user = system = 0; }
};
inline std::string format(const cpu_times& t) { return " " + std::to_string(t.wall * 1e-9) + "s wall"; }
class cpu_timer {
public:
    cpu_timer() { start(); }
    void start() { m_stopped = false; m_base = {}; m_t0 = std::chrono::steady_clock::now(); }
    void stop() { if (!m_stopped) { m_acc = elapsed(); m_stopped = true; } }
    void resume() { if (m_stopped) { m_base = m_acc; m_stopped = false; m_t0 = std::chrono::steady_clock::now(); } }
    bool is_stopped() const { return m_stopped; }
    cpu_times elapsed() const {
        if (m_stopped) return m_acc;
        auto ns = std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - m_t0).count();
        cpu_times t; t.wall = m_base.wall + ns; t.user = t.wall; t.system = 0; return t;
    }
    std::string format() const { return boost::timer::format(elapsed()); }
private:
    std::chrono::steady_clock::time_point m_t0;
    cpu_times m_acc{}, m_base{};
    bool m_stopped = false;
};
} // namespace timer
} // namespace boost
