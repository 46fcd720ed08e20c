// Build shim (test infrastructure only): the silver_bullets library is not installed.  The reference's
// worker and controller interfaces derive from silver_bullets::Factory<Interface> (a registry of named
// implementations); the adapter checks only need the base class to exist.
#pragma once
namespace silver_bullets {
template <class Interface> struct Factory {
    virtual ~Factory() = default;
};
} // namespace silver_bullets
