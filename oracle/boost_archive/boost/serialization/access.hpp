// TEST INFRASTRUCTURE ONLY.  Stand-in for Boost.Serialization's `access`,
// enough for the reference's GPU tool to load its inter.dat through the
// text-archive reader in boost/archive/text_iarchive.hpp of this directory.
#ifndef GLS_ARCHIVE_STUB_ACCESS
#define GLS_ARCHIVE_STUB_ACCESS
namespace boost {
namespace serialization {
class access {
public:
    template <class A, class T> static void serialize(A &a, T &t, unsigned version) { t.serialize(a, version); }
};
}  // namespace serialization
}  // namespace boost
#endif
