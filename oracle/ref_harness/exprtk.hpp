/*
 * Project-written stand-in for the third-party exprtk header (not vendored in
 * the reference, version unpinned).  The reference's Rietkerk and MultiSp
 * sources include <exprtk.hpp> only for their initial-frame builders; the
 * oracle harnesses never call those, so every member here aborts if reached.
 * TEST INFRASTRUCTURE ONLY.
 */
#pragma once
#include <string>
#include <vector>
#include <cstdlib>
#include <cstdio>
namespace exprtk {
[[noreturn]] inline void stub_abort(const char* w){ std::fprintf(stderr,"exprtk stub called: %s\n",w); std::abort(); }
template <typename T> class symbol_table {
public:
  bool add_variable(const std::string&, T&, bool = false){ stub_abort("add_variable"); }
  template <typename S> std::size_t get_variable_list(S&) const { stub_abort("get_variable_list"); }
  bool symbol_exists(const std::string&) const { stub_abort("symbol_exists"); }
  T* get_variable(const std::string&) const { stub_abort("get_variable"); }
  bool add_constants(){ stub_abort("add_constants"); }
  bool remove_variable(const std::string&, bool = false){ stub_abort("remove_variable"); }
};
template <typename T> class expression {
public:
  void register_symbol_table(symbol_table<T>&){ stub_abort("register_symbol_table"); }
  T value() const { stub_abort("value"); }
};
template <typename T> class parser {
public:
  bool compile(const std::string&, expression<T>&){ stub_abort("compile"); }
  std::string error() const { stub_abort("error"); }
};
}
