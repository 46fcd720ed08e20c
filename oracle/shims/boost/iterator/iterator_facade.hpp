// Oracle build shim: a small CRTP iterator base covering the subset of
// boost::iterator_facade that the reference headers use (dereference,
// increment, decrement, advance, distance_to, equal).
#pragma once
#include <cstddef>
#include <iterator>
#include <type_traits>
namespace boost {
struct forward_traversal_tag {};
struct bidirectional_traversal_tag {};
struct random_access_traversal_tag {};
struct iterator_core_access {};
namespace shim_detail {
template <class Tag> struct std_tag { using type = std::forward_iterator_tag; };
template <> struct std_tag<random_access_traversal_tag> { using type = std::random_access_iterator_tag; };
template <> struct std_tag<bidirectional_traversal_tag> { using type = std::bidirectional_iterator_tag; };
template <> struct std_tag<std::random_access_iterator_tag> { using type = std::random_access_iterator_tag; };
template <> struct std_tag<std::bidirectional_iterator_tag> { using type = std::bidirectional_iterator_tag; };
template <class T> struct arrow_proxy {
    T v;
    T* operator->() { return &v; }
};
}
template <class Derived, class Value, class CategoryOrTraversal,
          class Reference = Value&, class Difference = std::ptrdiff_t>
class iterator_facade {
public:
    using value_type = std::remove_const_t<Value>;
    using reference = Reference;
    using difference_type = Difference;
    using pointer = std::conditional_t<std::is_reference_v<Reference>,
                                       std::add_pointer_t<std::remove_reference_t<Reference>>,
                                       shim_detail::arrow_proxy<value_type>>;
    using iterator_category = typename shim_detail::std_tag<CategoryOrTraversal>::type;

    reference operator*() const { return self().dereference(); }
    auto operator->() const {
        if constexpr (std::is_reference_v<Reference>)
            return &self().dereference();
        else
            return shim_detail::arrow_proxy<value_type>{self().dereference()};
    }
    Derived& operator++() { self().increment(); return self(); }
    Derived operator++(int) { Derived t = self(); self().increment(); return t; }
    Derived& operator--() { self().decrement(); return self(); }
    Derived operator--(int) { Derived t = self(); self().decrement(); return t; }
    Derived& operator+=(difference_type n) { self().advance(n); return self(); }
    Derived& operator-=(difference_type n) { self().advance(-n); return self(); }
    Derived operator+(difference_type n) const { Derived t = self(); t.advance(n); return t; }
    Derived operator-(difference_type n) const { Derived t = self(); t.advance(-n); return t; }
    difference_type operator-(const Derived& that) const { return that.distance_to(self()); }
    reference operator[](difference_type n) const { return *(self() + n); }
    friend bool operator==(const Derived& a, const Derived& b) { return a.equal(b); }
    friend bool operator!=(const Derived& a, const Derived& b) { return !a.equal(b); }
    friend bool operator<(const Derived& a, const Derived& b) { return a.distance_to(b) > 0; }
private:
    Derived& self() { return *static_cast<Derived*>(this); }
    const Derived& self() const { return *static_cast<const Derived*>(this); }
};
} // namespace boost
