// TEST INFRASTRUCTURE ONLY.  A reader of Boost.Serialization text archives
// for the types the reference's `inter` archives (src/simulate.cu:46-104 and
// the classes it holds), so that the reference's GPU tool can be built and
// timed here without Boost.  It follows the same published rules as the
// tools' own archive code (gate-level-simulator_gb300/host/boost_inter.cpp):
//   * header: the string "serialization::archive" ("22 " + text), then the
//     library version;
//   * a class object whose type is seen for the first time is preceded by
//     its tracking flag and version; every type takes a class number at its
//     first use; a tracked type's objects carry an object number;
//   * arithmetic and enum values are single tokens; a string is its length,
//     one delimiter and its bytes;
//   * collections of arithmetic values carry no class information, every
//     other collection (of enums too, and std::pair) is a class; a
//     collection is its count, its item version and its elements; a map's
//     elements are pairs;
//   * a pointer is its target type's class number (-1: null), then (first
//     time) tracking and version, then the object number and the object.
// A malformed archive throws std::runtime_error.
#ifndef GLS_ARCHIVE_STUB_IARCHIVE
#define GLS_ARCHIVE_STUB_IARCHIVE
#include <cerrno>
#include <cstdlib>
#include <deque>
#include <istream>
#include <iterator>
#include <map>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <typeindex>
#include <unordered_map>
#include <utility>
#include <vector>
#include <boost/serialization/access.hpp>

namespace boost {
namespace archive {

class text_iarchive {
public:
    explicit text_iarchive(std::istream &is) : buf_(std::istreambuf_iterator<char>(is), std::istreambuf_iterator<char>())
    {
        std::string sig;
        load(sig);
        if (sig != "serialization::archive") throw std::runtime_error("not a Boost text archive");
        unsigned library_version = 0;
        load(library_version);
    }
    template <class T> text_iarchive &operator&(T &x)
    {
        load(x);
        return *this;
    }
    template <class T> text_iarchive &operator>>(T &x)
    {
        load(x);
        return *this;
    }

private:
    template <class T> struct is_primitive : std::integral_constant<bool, std::is_arithmetic<T>::value> {};

    std::string buf_;
    size_t at_ = 0;
    std::unordered_map<std::type_index, int> id_;
    std::vector<char> tracked_;
    std::vector<void *> objects_;   // objects read through pointers, by object number

    [[noreturn]] void fail(const std::string &m) { throw std::runtime_error("archive: " + m); }
    std::string word()
    {
        while (at_ < buf_.size() && isspace((unsigned char)buf_[at_])) ++at_;
        const size_t b = at_;
        while (at_ < buf_.size() && !isspace((unsigned char)buf_[at_])) ++at_;
        if (b == at_) fail("ends early");
        return buf_.substr(b, at_ - b);
    }
    long long integer()
    {
        const std::string w = word();
        char *end = nullptr;
        errno = 0;
        const long long v = w[0] == '-' ? strtoll(w.c_str(), &end, 10) : (long long)strtoull(w.c_str(), &end, 10);
        if (*end || errno) fail("bad integer '" + w + "'");
        return v;
    }
    bool first_use(std::type_index k)
    {
        if (id_.count(k)) return false;
        id_.emplace(k, (int)tracked_.size());
        tracked_.push_back(0);
        return true;
    }
    void class_info(std::type_index k)
    {
        const long long tracking = integer();
        integer();   // class version
        tracked_[id_[k]] = tracking != 0;
    }
    // a class-typed object: class information at its type's first use, an
    // object number when the type is tracked, then the body
    template <class T, class F> void object(bool info, F &&body)
    {
        const std::type_index k(typeid(T));
        if (first_use(k) && info) class_info(k);
        if (tracked_[id_[k]]) integer();
        body();
    }
    size_t count_and_version()
    {
        const long long n = integer();
        integer();   // item version
        if (n < 0 || (unsigned long long)n > buf_.size() - at_) fail("bad collection count");
        return (size_t)n;
    }

    template <class T> typename std::enable_if<std::is_floating_point<T>::value>::type load(T &x)
    {
        const std::string w = word();
        char *end = nullptr;
        x = (T)strtod(w.c_str(), &end);
        if (*end) fail("bad number '" + w + "'");
    }
    template <class T> typename std::enable_if<std::is_integral<T>::value>::type load(T &x) { x = (T)integer(); }
    template <class T> typename std::enable_if<std::is_enum<T>::value>::type load(T &x) { x = (T)integer(); }
    void load(std::string &s)
    {
        const long long n = integer();
        if (n < 0) fail("bad string length");
        if (n > 0) {
            ++at_;   // the one delimiter before the bytes
            if ((unsigned long long)n > buf_.size() - at_) fail("string runs past the end");
            s.assign(buf_, at_, (size_t)n);
            at_ += (size_t)n;
        } else {
            s.clear();
        }
    }
    template <class T> void load(std::vector<T> &v)
    {
        object<std::vector<T>>(!is_primitive<T>::value, [&] {
            v.assign(count_and_version(), T());
            for (auto &x : v) load(x);
        });
    }
    template <class T> void load(std::deque<T> &v)
    {
        object<std::deque<T>>(!is_primitive<T>::value, [&] {
            v.assign(count_and_version(), T());
            for (auto &x : v) load(x);
        });
    }
    template <class K, class V> void load(std::map<K, V> &m)
    {
        object<std::map<K, V>>(true, [&] {
            const size_t n = count_and_version();
            m.clear();
            for (size_t i = 0; i < n; ++i) {
                K k{};
                V v{};
                object<std::pair<const K, V>>(true, [&] {
                    load(k);
                    load(v);
                });
                m.emplace(std::move(k), std::move(v));
            }
        });
    }
    template <class T> void load(T *&p)
    {
        const long long cid = integer();
        if (cid == -1) {
            p = nullptr;
            return;
        }
        const std::type_index k(typeid(T));
        const auto it = id_.find(k);
        if (it == id_.end()) {
            if (cid != (long long)tracked_.size()) fail("unexpected class number");
            first_use(k);
            class_info(k);
        } else if (it->second != cid) {
            fail("pointer class number does not match its type");
        }
        if (!tracked_[id_[k]]) {
            p = new T();
            load_body(*p);
            return;
        }
        const long long oid = integer();
        if (oid >= 0 && (size_t)oid < objects_.size()) {
            p = static_cast<T *>(objects_[(size_t)oid]);
            return;
        }
        if (oid != (long long)objects_.size()) fail("object number out of sequence");
        p = new T();
        objects_.push_back(p);
        load_body(*p);
    }
    // a pointed-to object: its class information came with the pointer
    template <class T> void load_body(std::deque<T> &v)
    {
        v.assign(count_and_version(), T());
        for (auto &x : v) load(x);
    }
    template <class T> void load_body(std::vector<T> &v)
    {
        v.assign(count_and_version(), T());
        for (auto &x : v) load(x);
    }
    template <class T> typename std::enable_if<std::is_class<T>::value>::type load_body(T &x)
    {
        boost::serialization::access::serialize(*this, x, 0u);
    }
    // every other class: its own serialize()
    template <class T>
    typename std::enable_if<std::is_class<T>::value && !std::is_same<T, std::string>::value>::type load(T &x)
    {
        object<T>(true, [&] { boost::serialization::access::serialize(*this, x, 0u); });
    }
};

}  // namespace archive
}  // namespace boost
#endif
