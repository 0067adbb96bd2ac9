// Stand-in for the boost names that src/base/common.h imports; the compiled
// reference math files use none of them.
#pragma once
#include <memory>
#include <unordered_map>
#include <string>
namespace boost {
template <typename T> using shared_ptr = std::shared_ptr<T>;
template <typename T> using scoped_ptr = std::unique_ptr<T>;
template <typename K, typename V> using unordered_map = std::unordered_map<K, V>;
struct noncopyable { noncopyable() = default; noncopyable(const noncopyable&) = delete; };
struct format { explicit format(const char*) {} };
template <typename T, typename S> T lexical_cast(const S&) { return T(); }
template <typename T> struct irange_t { T a, b; };
template <typename T> irange_t<T> irange(T a, T b) { return irange_t<T>{a, b}; }
}
