// Type-checking stand-in for the XLA FFI C++ binding API, used only by
// tests/test_jax_ffi_shim.py to compile tensorf-jax_gb300/csrc/jax/tvm_jax_ffi.cc on
// a machine without jaxlib. It declares the names the shim uses (Buffer,
// ResultBuffer, Error, Ffi::Bind, XLA_FFI_DEFINE_HANDLER_SYMBOL) with the same shapes,
// and it checks at compile time what a real binding would reject: that each handler
// can be called with the binding's context, argument, result and attribute types, in
// the binding's order. Nothing here runs.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <type_traits>

namespace xla::ffi {

enum class DataType { F32, U8 };
inline constexpr DataType F32 = DataType::F32;
inline constexpr DataType U8 = DataType::U8;

template <DataType T> struct NativeType;
template <> struct NativeType<DataType::F32> { using type = float; };
template <> struct NativeType<DataType::U8> { using type = std::uint8_t; };

struct Span {
  const std::int64_t* data;
  std::size_t size;
  std::int64_t operator[](std::size_t i) const { return data[i]; }
};

template <DataType T>
class Buffer {
 public:
  using value_type = typename NativeType<T>::type;
  value_type* typed_data() const { return nullptr; }
  std::size_t element_count() const { return 0; }
  std::size_t size_bytes() const { return 0; }
  Span dimensions() const { return Span{nullptr, 0}; }
};

template <typename T>
class Result {
 public:
  T* operator->() { return &value_; }
  T& operator*() { return value_; }

 private:
  T value_;
};

template <DataType T> using ResultBuffer = Result<Buffer<T>>;

enum class ErrorCode { kOk, kInvalidArgument, kInternal };

class Error {
 public:
  Error() = default;
  Error(ErrorCode code, std::string message) : code_(code), message_(std::move(message)) {}
  static Error Success() { return Error(); }
  bool success() const { return code_ == ErrorCode::kOk; }
  bool failure() const { return !success(); }

 private:
  ErrorCode code_ = ErrorCode::kOk;
  std::string message_;
};

template <typename T> struct PlatformStream {};

// What a bound entry turns into as a handler parameter.
template <typename T> struct Decoded { using type = T; };
template <typename S> struct Decoded<PlatformStream<S>> { using type = S; };
template <typename... Ts>
struct Binding {
  template <typename T> constexpr Binding<Ts..., T> Ctx() const { return {}; }
  template <typename T> constexpr Binding<Ts..., T> Arg() const { return {}; }
  template <typename T> constexpr Binding<Ts..., Result<T>> Ret() const { return {}; }
  template <typename T> constexpr Binding<Ts..., T> Attr(const char*) const { return {}; }
};

struct Ffi {
  static constexpr Binding<> Bind() { return {}; }
};

template <typename... Ts> struct TypeList {};

// The handler's parameter types must be exactly the decoded binding entries, in order,
// and it must return Error: no conversions, as the real decoder allows none.
template <typename... Ps, typename... Ts>
constexpr bool handler_matches(Error (*)(Ps...), Binding<Ts...>) {
  return std::is_same_v<TypeList<Ps...>, TypeList<typename Decoded<Ts>::type...>>;
}

}  // namespace xla::ffi

#define XLA_FFI_DEFINE_HANDLER_SYMBOL(name, fn, binding)                                        \
  static_assert(::xla::ffi::handler_matches(&fn, binding), #name ": handler does not match its binding"); \
  extern "C" void* name() { return reinterpret_cast<void*>(&fn); }
