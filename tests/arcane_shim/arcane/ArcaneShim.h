// Stand-ins for the few Arcane types the GB300 linear-system service uses, so
// that it compiles and runs without Arcane (which needs .NET, MPI and HYPRE).
// Test infrastructure: only the signatures the service touches, with the
// meaning Arcane gives them (Real = double, Byte = unsigned char, DoF local
// ids = Int32, mesh variables = one value per item).
#pragma once

#include <cstdint>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace Arcane
{
using Real = double;
using Int32 = std::int32_t;
using Int64 = std::int64_t;
using Byte = unsigned char;
using Bool = bool;

class String
{
 public:
  String() = default;
  String(const char* s) : m_s(s) {}
  String(std::string s) : m_s(std::move(s)) {}
  friend String operator+(const String& a, const char* b) { return String(a.m_s + b); }
  const std::string& str() const { return m_s; }

 private:
  std::string m_s;
};

//! DoF local id (ItemLocalIdT<DoF>).
class DoFLocalId
{
 public:
  constexpr explicit DoFLocalId(Int32 id) : m_id(id) {}
  constexpr Int32 localId() const { return m_id; }

 private:
  Int32 m_id;
};

class ITraceMng
{};

class IItemFamily
{
 public:
  explicit IItemFamily(Int32 nb_item) : m_nb_item(nb_item) {}
  Int32 nbItem() const { return m_nb_item; }
  ITraceMng* traceMng() { return &m_trace; }

 private:
  Int32 m_nb_item;
  ITraceMng m_trace;
};

class ISubDomain
{};
class CommandLineArguments
{};
class Runner
{};

template <class T>
class ArrayView
{
 public:
  ArrayView(T* p, Int64 n) : m_p(p), m_n(n) {}
  T* data() const { return m_p; }
  Int64 size() const { return m_n; }
  T& operator[](Int64 i) const { return m_p[i]; }

 private:
  T* m_p;
  Int64 m_n;
};

template <class T>
class Span
{
 public:
  Span() = default;
  Span(T* p, Int64 n) : m_p(p), m_n(n) {}
  T* data() const { return m_p; }
  Int64 size() const { return m_n; }
  T& operator[](Int64 i) const { return m_p[i]; }

 private:
  T* m_p = nullptr;
  Int64 m_n = 0;
};
template <class T>
using SmallSpan = Span<T>;

//! A scalar DoF variable (MeshVariableScalarRefT<DoF, T>), host storage.
template <class T>
class VariableDoF
{
 public:
  VariableDoF(IItemFamily* family, const String&) : m_v(family->nbItem()) {}
  ArrayView<T> asArray() { return ArrayView<T>(m_v.data(), (Int64)m_v.size()); }
  void fill(T v) { std::fill(m_v.begin(), m_v.end(), v); }
  T& operator[](DoFLocalId i) { return m_v[i.localId()]; }

 private:
  std::vector<T> m_v;
};
template <>
class VariableDoF<bool>
{
 public:
  VariableDoF(IItemFamily* family, const String&) : m_v(family->nbItem()) {}
  ArrayView<bool> asArray() { return ArrayView<bool>(reinterpret_cast<bool*>(m_v.data()), (Int64)m_v.size()); }
  void fill(bool v) { std::fill(m_v.begin(), m_v.end(), (unsigned char)v); }
  bool& operator[](DoFLocalId i) { return reinterpret_cast<bool&>(m_v[i.localId()]); }

 private:
  std::vector<unsigned char> m_v;   // one byte per item, as Arcane stores Bool
};
using VariableDoFReal = VariableDoF<Real>;
using VariableDoFByte = VariableDoF<Byte>;
using VariableDoFBool = VariableDoF<bool>;

class TraceAccessor
{
 public:
  explicit TraceAccessor(ITraceMng*) {}
  std::ostream& info() const { return std::clog; }
};

class FatalErrorException : public std::runtime_error
{
  using std::runtime_error::runtime_error;
};
class NotImplementedException : public std::logic_error
{
  using std::logic_error::logic_error;
};
class ArgumentException : public std::invalid_argument
{
  using std::invalid_argument::invalid_argument;
};

namespace shim
{
  // "{0} {1}" formatting of ARCANE_FATAL / ARCANE_THROW
  inline void format_rest(std::ostringstream&, const std::string& f, size_t pos, int) { (void)f; (void)pos; }
  template <class A, class... R>
  void format_rest(std::ostringstream& o, const std::string& f, size_t pos, int k, const A& a, const R&... r)
  {
    const std::string tag = "{" + std::to_string(k) + "}";
    const size_t at = f.find(tag, pos);
    if (at == std::string::npos) {
      o << f.substr(pos);
      return;
    }
    o << f.substr(pos, at - pos) << a;
    const size_t next = at + tag.size();
    if (sizeof...(R) == 0)
      o << f.substr(next);
    else
      format_rest(o, f, next, k + 1, r...);
  }
  template <class... A>
  std::string format(const char* f, const A&... a)
  {
    std::ostringstream o;
    if constexpr (sizeof...(A) == 0)
      o << f;
    else
      format_rest(o, std::string(f), 0, 0, a...);
    return o.str();
  }
} // namespace shim

} // namespace Arcane

#define ARCANE_FATAL(...) throw ::Arcane::FatalErrorException(::Arcane::shim::format(__VA_ARGS__))
#define ARCANE_THROW(exc, ...) throw ::Arcane::exc(::Arcane::shim::format(__VA_ARGS__))
