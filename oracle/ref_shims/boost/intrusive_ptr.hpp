/* Minimal intrusive_ptr with the surface the reference uses (oracle build
 * only).  Reference counting calls intrusive_ptr_add_ref/_release found by
 * argument-dependent lookup, like the Boost original. */
#ifndef SKW_REF_SHIM_INTRUSIVE_PTR_HPP
#define SKW_REF_SHIM_INTRUSIVE_PTR_HPP
#include <cstddef>
#include <functional>

namespace boost {

template <class T>
class intrusive_ptr {
 public:
  typedef T element_type;
  intrusive_ptr() : p_(nullptr) {}
  intrusive_ptr(T *p, bool add_ref = true) : p_(p) {
    if (p_ && add_ref) intrusive_ptr_add_ref(p_);
  }
  intrusive_ptr(const intrusive_ptr &o) : p_(o.p_) {
    if (p_) intrusive_ptr_add_ref(p_);
  }
  template <class U>
  intrusive_ptr(const intrusive_ptr<U> &o) : p_(o.get()) {
    if (p_) intrusive_ptr_add_ref(p_);
  }
  intrusive_ptr(intrusive_ptr &&o) noexcept : p_(o.p_) { o.p_ = nullptr; }
  ~intrusive_ptr() {
    if (p_) intrusive_ptr_release(p_);
  }
  intrusive_ptr &operator=(const intrusive_ptr &o) {
    intrusive_ptr(o).swap(*this);
    return *this;
  }
  intrusive_ptr &operator=(intrusive_ptr &&o) noexcept {
    intrusive_ptr(static_cast<intrusive_ptr &&>(o)).swap(*this);
    return *this;
  }
  template <class U>
  intrusive_ptr &operator=(const intrusive_ptr<U> &o) {
    intrusive_ptr(o).swap(*this);
    return *this;
  }
  intrusive_ptr &operator=(T *p) {
    intrusive_ptr(p).swap(*this);
    return *this;
  }
  void reset() { intrusive_ptr().swap(*this); }
  void reset(T *p) { intrusive_ptr(p).swap(*this); }
  T *get() const { return p_; }
  T &operator*() const { return *p_; }
  T *operator->() const { return p_; }
  explicit operator bool() const { return p_ != nullptr; }
  bool operator!() const { return p_ == nullptr; }
  void swap(intrusive_ptr &o) {
    T *t = p_;
    p_ = o.p_;
    o.p_ = t;
  }

 private:
  T *p_;
};

template <class T, class U>
bool operator==(const intrusive_ptr<T> &a, const intrusive_ptr<U> &b) { return a.get() == b.get(); }
template <class T, class U>
bool operator!=(const intrusive_ptr<T> &a, const intrusive_ptr<U> &b) { return a.get() != b.get(); }
template <class T, class U>
bool operator==(const intrusive_ptr<T> &a, U *b) { return a.get() == b; }
template <class T, class U>
bool operator!=(const intrusive_ptr<T> &a, U *b) { return a.get() != b; }
template <class T, class U>
bool operator==(T *a, const intrusive_ptr<U> &b) { return a == b.get(); }
template <class T, class U>
bool operator!=(T *a, const intrusive_ptr<U> &b) { return a != b.get(); }
/* Comparisons against NULL (an integer constant with g++'s __null). */
template <class T>
bool operator==(const intrusive_ptr<T> &a, long z) { return a.get() == (T *)z; }
template <class T>
bool operator!=(const intrusive_ptr<T> &a, long z) { return a.get() != (T *)z; }
template <class T>
bool operator==(long z, const intrusive_ptr<T> &a) { return a.get() == (T *)z; }
template <class T>
bool operator!=(long z, const intrusive_ptr<T> &a) { return a.get() != (T *)z; }
template <class T>
bool operator==(const intrusive_ptr<T> &a, std::nullptr_t) { return a.get() == nullptr; }
template <class T>
bool operator!=(const intrusive_ptr<T> &a, std::nullptr_t) { return a.get() != nullptr; }
template <class T>
bool operator<(const intrusive_ptr<T> &a, const intrusive_ptr<T> &b) { return std::less<T *>()(a.get(), b.get()); }
template <class T, class U>
intrusive_ptr<T> static_pointer_cast(const intrusive_ptr<U> &p) { return intrusive_ptr<T>(static_cast<T *>(p.get())); }
template <class T, class U>
intrusive_ptr<T> dynamic_pointer_cast(const intrusive_ptr<U> &p) { return intrusive_ptr<T>(dynamic_cast<T *>(p.get())); }
template <class T, class U>
intrusive_ptr<T> const_pointer_cast(const intrusive_ptr<U> &p) { return intrusive_ptr<T>(const_cast<T *>(p.get())); }

}  // namespace boost

#endif
