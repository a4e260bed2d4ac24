/*
 * cu_memory.hpp -- reference-counted device / host / pitched containers with
 * the semantics of the reference's cu_memory.hpp:46-640:
 *   - copies share the buffer and bump a reference count;
 *   - create() is a no-op when the size is unchanged;
 *   - the (ptr, size) constructors wrap caller memory without owning it;
 *   - upload() / download() are synchronous;
 *   - cu_memory_2d / cu_array_2d are pitched (cudaMallocPitch).
 * CUDA failures throw mcg_cuda_error (the reference aborts the process).
 */
#ifndef MCG_CU_MEMORY_HPP
#define MCG_CU_MEMORY_HPP

#include <stddef.h>

#include <stdexcept>
#include <string>
#include <vector>

#if defined(__CUDACC__)
#define MCG_HOSTDEV __host__ __device__
#else
#define MCG_HOSTDEV
#endif

class mcg_cuda_error : public std::runtime_error {
public:
    mcg_cuda_error(const std::string &what, int code) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

/* ---- kernel-side views (cu_memory.hpp:46-89) ---- */
template <typename T>
struct cu_ptr {
    typedef T elem_type;
    static const size_t elem_size_ = sizeof(elem_type);
    T *data;
    MCG_HOSTDEV cu_ptr() : data(0) {}
    MCG_HOSTDEV cu_ptr(T *data_arg) : data(data_arg) {}
    MCG_HOSTDEV size_t elem_size() const { return elem_size_; }
    MCG_HOSTDEV operator T *() { return data; }
    MCG_HOSTDEV operator const T *() const { return data; }
};

template <typename T>
struct ptr_size : public cu_ptr<T> {
    MCG_HOSTDEV ptr_size() : size(0) {}
    MCG_HOSTDEV ptr_size(T *data_arg, size_t size_arg) : cu_ptr<T>(data_arg), size(size_arg) {}
    size_t size;
};

template <typename T>
struct ptr_step : public cu_ptr<T> {
    MCG_HOSTDEV ptr_step() : step(0) {}
    MCG_HOSTDEV ptr_step(T *data_arg, size_t step_arg) : cu_ptr<T>(data_arg), step(step_arg) {}
    size_t step; /* bytes between rows */
    MCG_HOSTDEV T *ptr(int y = 0) { return (T *)((char *)cu_ptr<T>::data + y * step); }
    MCG_HOSTDEV const T *ptr(int y = 0) const { return (const T *)((const char *)cu_ptr<T>::data + y * step); }
};

template <typename T>
struct ptr_step_size : public ptr_step<T> {
    MCG_HOSTDEV ptr_step_size() : cols(0), rows(0) {}
    MCG_HOSTDEV ptr_step_size(int rows_arg, int cols_arg, T *data_arg, size_t step_arg)
        : ptr_step<T>(data_arg, step_arg), cols(cols_arg), rows(rows_arg) {}
    int cols;
    int rows;
};

/* ---- untyped containers ---- */
class cu_memory {
public:
    cu_memory();
    ~cu_memory();
    explicit cu_memory(size_t size_bytes_arg);
    cu_memory(void *ptr_arg, size_t size_bytes_arg); /* non-owning */
    cu_memory(const cu_memory &other_arg);
    cu_memory &operator=(const cu_memory &other_arg);
    void create(size_t size_bytes_arg);
    void release();
    void copy_to(cu_memory &other) const;
    void upload(const void *host_ptr_arg, size_t size_bytes_arg);
    void download(void *host_ptr_arg) const;
    void swap(cu_memory &other_arg);
    template <class T> T *ptr() { return (T *)data_; }
    template <class T> const T *ptr() const { return (const T *)data_; }
    template <class U> operator ptr_size<U>() const {
        return ptr_size<U>((U *)data_, size_bytes_ / sizeof(U));
    }
    bool empty() const { return !data_; }
    size_t size_bytes() const { return size_bytes_; }

private:
    void *data_;
    size_t size_bytes_;
    int *refcount_;
};

class cu_memory_host {
public:
    cu_memory_host();
    ~cu_memory_host();
    explicit cu_memory_host(size_t size_bytes_arg);
    cu_memory_host(void *ptr_arg, size_t size_bytes_arg); /* non-owning */
    cu_memory_host(const cu_memory_host &other_arg);
    cu_memory_host &operator=(const cu_memory_host &other_arg);
    void create(size_t size_bytes_arg);
    void release();
    void copy_to(cu_memory_host &other) const;
    void upload(const void *ptr_arg, size_t size_bytes_arg); /* host -> host */
    void download(void *ptr_arg) const;
    void swap(cu_memory_host &other_arg);
    template <class T> T *ptr() { return (T *)data_; }
    template <class T> const T *ptr() const { return (const T *)data_; }
    bool empty() const { return !data_; }
    size_t size_bytes() const { return size_bytes_; }

private:
    void *data_;
    size_t size_bytes_;
    int *refcount_;
};

class cu_memory_2d {
public:
    cu_memory_2d();
    ~cu_memory_2d();
    cu_memory_2d(int rows_arg, int colsBytes_arg);
    cu_memory_2d(int rows_arg, int colsBytes_arg, void *data_arg, size_t step_arg); /* non-owning */
    cu_memory_2d(const cu_memory_2d &other_arg);
    cu_memory_2d &operator=(const cu_memory_2d &other_arg);
    void create(int rows_arg, int colsBytes_arg);
    void release();
    void copy_to(cu_memory_2d &other) const;
    void upload(const void *host_ptr_arg, size_t host_step_arg, int rows_arg, int colsBytes_arg);
    void download(void *host_ptr_arg, size_t host_step_arg) const;
    void swap(cu_memory_2d &other_arg);
    template <class T> T *ptr(int y_arg = 0) { return (T *)((char *)data_ + y_arg * step_); }
    template <class T> const T *ptr(int y_arg = 0) const { return (const T *)((const char *)data_ + y_arg * step_); }
    template <class U> operator ptr_step<U>() const { return ptr_step<U>((U *)data_, step_); }
    template <class U> operator ptr_step_size<U>() const {
        return ptr_step_size<U>(rows_, (int)(colsBytes_ / sizeof(U)), (U *)data_, step_);
    }
    bool empty() const { return !data_; }
    int colsBytes() const { return colsBytes_; }
    int rows() const { return rows_; }
    size_t step() const { return step_; }

private:
    void *data_;
    size_t step_;
    int colsBytes_;
    int rows_;
    int *refcount_;
};

/* ---- typed containers ---- */
template <class T>
class cu_array : public cu_memory {
public:
    typedef T type;
    enum { elem_size = sizeof(T) };
    cu_array() {}
    explicit cu_array(size_t size) : cu_memory(size * elem_size) {}
    cu_array(T *ptr, size_t size) : cu_memory(ptr, size * elem_size) {}
    cu_array(const cu_array &other) : cu_memory(other) {}
    cu_array &operator=(const cu_array &other) { cu_memory::operator=(other); return *this; }
    void create(size_t size) { cu_memory::create(size * elem_size); }
    void release() { cu_memory::release(); }
    void copy_to(cu_array &other) const { cu_memory::copy_to(other); }
    void upload(const T *host_ptr, size_t size) { cu_memory::upload(host_ptr, size * elem_size); }
    void download(T *host_ptr) const { cu_memory::download(host_ptr); }
    template <class A> void upload(const std::vector<T, A> &data) { upload(&data[0], data.size()); }
    template <class A> void download(std::vector<T, A> &data) const {
        data.resize(size());
        if (!data.empty()) download(&data[0]);
    }
    void swap(cu_array &other_arg) { cu_memory::swap(other_arg); }
    T *ptr() { return cu_memory::ptr<T>(); }
    const T *ptr() const { return cu_memory::ptr<T>(); }
    operator T *() { return ptr(); }
    operator const T *() const { return ptr(); }
    size_t size() const { return size_bytes() / elem_size; }
};

template <class T>
class cu_array_host : public cu_memory_host {
public:
    typedef T type;
    enum { elem_size = sizeof(T) };
    cu_array_host() {}
    explicit cu_array_host(size_t size) : cu_memory_host(size * elem_size) {}
    cu_array_host(T *ptr, size_t size) : cu_memory_host(ptr, size * elem_size) {}
    cu_array_host(const cu_array_host &other) : cu_memory_host(other) {}
    cu_array_host &operator=(const cu_array_host &other) { cu_memory_host::operator=(other); return *this; }
    void create(size_t size) { cu_memory_host::create(size * elem_size); }
    void release() { cu_memory_host::release(); }
    void upload(const T *host_ptr, size_t size) { cu_memory_host::upload(host_ptr, size * elem_size); }
    void download(T *host_ptr) const { cu_memory_host::download(host_ptr); }
    void swap(cu_array_host &other_arg) { cu_memory_host::swap(other_arg); }
    T *ptr() { return cu_memory_host::ptr<T>(); }
    const T *ptr() const { return cu_memory_host::ptr<T>(); }
    operator T *() { return ptr(); }
    operator const T *() const { return ptr(); }
    size_t size() const { return size_bytes() / elem_size; }
};

template <class T>
class cu_array_2d : public cu_memory_2d {
public:
    typedef T type;
    enum { elem_size = sizeof(T) };
    cu_array_2d() {}
    cu_array_2d(int rows, int cols) : cu_memory_2d(rows, cols * elem_size) {}
    cu_array_2d(int rows, int cols, void *data, size_t step_bytes) : cu_memory_2d(rows, cols * elem_size, data, step_bytes) {}
    cu_array_2d(const cu_array_2d &other) : cu_memory_2d(other) {}
    cu_array_2d &operator=(const cu_array_2d &other) { cu_memory_2d::operator=(other); return *this; }
    void create(int rows, int cols) { cu_memory_2d::create(rows, cols * elem_size); }
    void release() { cu_memory_2d::release(); }
    void copy_to(cu_array_2d &other) const { cu_memory_2d::copy_to(other); }
    void upload(const void *host_ptr, size_t host_step, int rows, int cols) {
        cu_memory_2d::upload(host_ptr, host_step, rows, cols * elem_size);
    }
    void download(void *host_ptr, size_t host_step) const { cu_memory_2d::download(host_ptr, host_step); }
    void swap(cu_array_2d &other_arg) { cu_memory_2d::swap(other_arg); }
    T *ptr(int y = 0) { return cu_memory_2d::ptr<T>(y); }
    const T *ptr(int y = 0) const { return cu_memory_2d::ptr<T>(y); }
    operator T *() { return ptr(); }
    operator const T *() const { return ptr(); }
    int cols() const { return cu_memory_2d::colsBytes() / elem_size; }
    int rows() const { return cu_memory_2d::rows(); }
    size_t elem_step() const { return cu_memory_2d::step() / elem_size; }
};

#endif
