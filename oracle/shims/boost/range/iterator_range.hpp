// Oracle build shim: boost::iterator_range and make_iterator_range.
#pragma once
#include <iterator>
#include <cstddef>
namespace boost {
template <class It> class iterator_range {
public:
    iterator_range() = default;
    iterator_range(It b, It e) : m_b(b), m_e(e) {}
    template <class R> iterator_range(R& r) : m_b(std::begin(r)), m_e(std::end(r)) {}
    It begin() const { return m_b; }
    It end() const { return m_e; }
    bool empty() const { return m_b == m_e; }
    auto size() const { return std::distance(m_b, m_e); }
    decltype(auto) front() const { return *m_b; }
    decltype(auto) operator[](std::ptrdiff_t i) const { return m_b[i]; }
private:
    It m_b{}, m_e{};
};
template <class It> inline iterator_range<It> make_iterator_range(It b, It e) { return {b, e}; }
template <class R> inline auto make_iterator_range(R& r) { return iterator_range<decltype(std::begin(r))>(std::begin(r), std::end(r)); }
template <class It, class N> inline iterator_range<It> make_iterator_range_n(It b, N n) { return {b, b + n}; }
} // namespace boost
