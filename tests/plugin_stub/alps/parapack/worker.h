// Stand-ins for the few ALPS parapack types the worker plug-in of INTEGRATION.md uses, so that the
// plug-in's own source compiles and runs in the tests without ALPS: Parameters (ordered KEY =
// value pairs), ObservableSet (named series of pushed values), ODump / IDump (a byte buffer),
// mc_worker and the registration macro.  Only what the plug-in touches is here.
#pragma once
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

namespace alps {

class ParamValue {
public:
  explicit ParamValue(std::string s = std::string()) : s_(std::move(s)) {}
  const char* c_str() const { return s_.c_str(); }
  operator uint64_t() const { return std::strtoull(s_.c_str(), nullptr, 10); }
  operator double() const { return std::strtod(s_.c_str(), nullptr); }

private:
  std::string s_;
};

class Parameter {
public:
  Parameter(std::string k, std::string v) : k_(std::move(k)), v_(std::move(v)) {}
  std::string key() const { return k_; }
  ParamValue value() const { return ParamValue(v_); }

private:
  std::string k_, v_;
};

class Parameters {
public:
  typedef std::vector<Parameter>::const_iterator const_iterator;
  void set(const std::string& k, const std::string& v) { ps_.push_back(Parameter(k, v)); }
  const_iterator begin() const { return ps_.begin(); }
  const_iterator end() const { return ps_.end(); }
  bool defined(const std::string& k) const {
    for (const Parameter& p : ps_)
      if (p.key() == k) return true;
    return false;
  }
  ParamValue operator[](const std::string& k) const {
    for (const Parameter& p : ps_)
      if (p.key() == k) return p.value();
    return ParamValue();
  }

private:
  std::vector<Parameter> ps_;
};

class RealObservable {
public:
  explicit RealObservable(const std::string& name) : name(name) {}
  std::string name;
};

class ObservableSet {
public:
  class Series {
  public:
    explicit Series(std::vector<double>* v) : v_(v) {}
    Series& operator<<(double x) {
      v_->push_back(x);
      return *this;
    }

  private:
    std::vector<double>* v_;
  };
  ObservableSet& operator<<(const RealObservable& o) {
    data[o.name];
    return *this;
  }
  Series operator[](const std::string& name) { return Series(&data.at(name)); }
  std::map<std::string, std::vector<double> > data;
};

class ODump {
public:
  template <class T>
  ODump& operator<<(const std::vector<T>& v) {
    *this << (uint64_t)v.size();
    const char* p = reinterpret_cast<const char*>(v.data());
    bytes.insert(bytes.end(), p, p + v.size() * sizeof(T));
    return *this;
  }
  template <class T>
  ODump& operator<<(const T& x) {
    const char* p = reinterpret_cast<const char*>(&x);
    bytes.insert(bytes.end(), p, p + sizeof(T));
    return *this;
  }
  std::vector<char> bytes;
};

class IDump {
public:
  explicit IDump(const std::vector<char>& b) : bytes(b) {}
  template <class T>
  IDump& operator>>(std::vector<T>& v) {
    uint64_t n = 0;
    *this >> n;
    v.resize(n);
    std::memcpy(v.data(), bytes.data() + at, n * sizeof(T));
    at += n * sizeof(T);
    return *this;
  }
  template <class T>
  IDump& operator>>(T& x) {
    std::memcpy(&x, bytes.data() + at, sizeof(T));
    at += sizeof(T);
    return *this;
  }
  std::vector<char> bytes;
  size_t at = 0;
};

namespace parapack {
class mc_worker {
public:
  explicit mc_worker(Parameters const&) {}
  virtual ~mc_worker() {}
};
template <class W>
class single_exchange_worker {};
}  // namespace parapack

}  // namespace alps

#define LG_STUB_CAT2(a, b) a##b
#define LG_STUB_CAT(a, b) LG_STUB_CAT2(a, b)
#define PARAPACK_REGISTER_ALGORITHM(worker, name) \
  typedef worker LG_STUB_CAT(lg_registered_, __COUNTER__);  \
  static_assert(sizeof(name) > 1, "algorithm name");
