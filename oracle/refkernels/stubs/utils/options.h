// Minimal stand-in for FSL's utils/options.h so that CUDIMOT's kernel files
// (which include cudimotoptions.h) compile without FSL. Only the device code
// of those files is used (compiled to cubins by oracle/refkernels/build_ref_kernels.py);
// the host classes below are never executed. TEST INFRASTRUCTURE.
#pragma once
#include <exception>
#include <string>
namespace Utilities {
enum ArgFlag { no_argument, requires_argument, optional_argument, requires_2_arguments,
               requires_3_arguments, requires_4_arguments, requires_5_arguments };
template <class T>
class Option {
 public:
  Option(const std::string&, const T& v, const std::string&, bool, ArgFlag) : v_(v) {}
  T value() const { return v_; }
  bool set() const { return false; }
  void set_value(const T& v) { v_ = v; }
 private:
  T v_;
};
template <class T>
class FmribOption : public Option<T> {
 public:
  using Option<T>::Option;
};
class OptionParser {
 public:
  OptionParser(const std::string&, const std::string&) {}
  template <class O> void add(O&) {}
  void usage() {}
};
class X_OptionError : public std::exception {};
}  // namespace Utilities
