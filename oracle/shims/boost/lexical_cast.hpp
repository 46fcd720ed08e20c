// Oracle build shim: boost::lexical_cast through string streams.
#pragma once
#include <sstream>
#include <string>
#include <stdexcept>
namespace boost {
template <class To, class From> inline To lexical_cast(const From& x) {
    std::stringstream s;
    s << x;
    To result;
    if (!(s >> result))
        throw std::runtime_error("lexical_cast failed");
    return result;
}
template <> inline std::string lexical_cast<std::string, std::string>(const std::string& x) { return x; }
} // namespace boost
