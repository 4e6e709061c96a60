// Stand-in for boost::throw_exception, for compiling the worker plug-in of INTEGRATION.md in the
// tests without Boost.
#pragma once
namespace boost {
template <class E>
[[noreturn]] void throw_exception(const E& e) {
  throw e;
}
}  // namespace boost
