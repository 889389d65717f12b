// Stub of the one Boost.Serialization name the reference headers need to
// compile without Boost (TEST INFRASTRUCTURE ONLY; no archive is ever read).
#ifndef GLS_STUB_BOOST_ACCESS
#define GLS_STUB_BOOST_ACCESS
namespace boost { namespace serialization { class access {}; } }
#endif
