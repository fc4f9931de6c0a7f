/*
 * gpu_array.h -- gpu_array_base / gpu_array<T> of the reference
 * (common/inc/gpu_array_base.h:17-123, common/inc/gpu_array.h:146-281) on CUDA
 * device memory.  The device pointer replaces cl_mem; the class never owns
 * host_ptr (gpu_array.h:272-276).  IN_GPU_USE_ONLY buffers persist until
 * dev_free(); TO_GPU / TO_GPU_AND_BACK buffers copy their host data at
 * construction (the reference copies at launch).  Errors throw
 * std::runtime_error where the reference aborts.
 */
#ifndef TDE_3DEYE_GPU_ARRAY_H
#define TDE_3DEYE_GPU_ARRAY_H

#include <stdexcept>
#include <string>

#include "tde_types.h"

void tde_cxx_throw_if(int status, const char *what);

class gpu_array_base {
  protected:
    void *device_ptr = nullptr;
    gpu_transfer_type data_transfer_direction = IN_GPU_USE_ONLY;
    gpu_data_type data_type = BUFFER_1D;
    dim3 sizes;
    unsigned int total_size = 0;
    bool need_to_prepare = false;
    gpu_mem_type mem_type = GLOBAL;

  public:
    gpu_array_base() {}
    virtual ~gpu_array_base();

    gpu_mem_type get_arg_mem_type() const { return mem_type; }
    void set_arg_mem_type(gpu_mem_type t) { mem_type = t; }
    void set_data_transfer_type(gpu_transfer_type t) { data_transfer_direction = t; }
    gpu_transfer_type get_data_transfer_type() const { return data_transfer_direction; }
    void set_data_type(gpu_data_type t) { data_type = t; }
    gpu_data_type get_data_type() const { return data_type; }
    void set_prepare_status(bool s) { need_to_prepare = s; }
    bool should_be_prepared() const { return need_to_prepare; }
    /* number of elements (the reference's total_size is x*y*z) */
    virtual unsigned int get_total_size() const { return total_size; }

    virtual void *get_host_ptr() = 0;
    virtual void set_host_ptr(void *ptr) = 0;
    virtual void set_host_ptr(void *ptr, dim3 &size) = 0;

    /* device address (the reference returned cl_mem *) */
    void **get_device_ptr() { return &device_ptr; }
    void *device() const { return device_ptr; }
    void set_device_ptr(void *p) { device_ptr = p; }

    void copy_to(gpu_array_base *dst);
    void memcpy_from_dev(void *host_dst);
    void memcpy_to_dev(void *host_src);
    virtual void memcpy_from_host(void *host_src) = 0;
    virtual void memcpy_to_host(void *host_dst) = 0;

    void dev_alloc();
    void dev_free();

    unsigned int width() const { return (unsigned)sizes.x; }
    unsigned int height() const { return (unsigned)sizes.y; }
    unsigned int depth() const { return (unsigned)sizes.z; }
    dim3 get_size() const { return sizes; }
    void set_size(const dim3 &s);
    virtual size_t elem_size() const = 0;
    size_t bytes() const { return (size_t)total_size * elem_size(); }
};

template <class T> class gpu_array : public gpu_array_base {
  public:
    gpu_array(T *host_data, dim3 host_data_size, gpu_transfer_type dir = TO_GPU) {
        host_ptr = host_data;
        set_size(host_data_size);
        data_transfer_direction = dir;
        dev_alloc();
        if (host_data && (dir == TO_GPU || dir == TO_GPU_AND_BACK)) memcpy_to_dev(host_data);
    }
    gpu_array(T *host_data, dim3 host_data_size, bool should_allocate_and_transfer,
              gpu_transfer_type dir = IN_GPU_USE_ONLY) {
        host_ptr = host_data;
        set_size(host_data_size);
        data_transfer_direction = dir;
        if (should_allocate_and_transfer) {
            dev_alloc();
            if (host_data) memcpy_to_dev(host_data);
        }
    }
    gpu_array(dim3 host_data_size, bool should_allocate = true, gpu_transfer_type dir = IN_GPU_USE_ONLY) {
        set_size(host_data_size);
        data_transfer_direction = dir;
        if (should_allocate) dev_alloc();
    }
    gpu_array(unsigned int n, bool should_allocate = true, gpu_transfer_type dir = IN_GPU_USE_ONLY)
        : gpu_array(dim3(n), should_allocate, dir) {}
    ~gpu_array() {}

    void *get_host_ptr() { return host_ptr; }
    T *get_host_ptr_impl() { return host_ptr; }
    void set_host_ptr(void *p) { host_ptr = static_cast<T *>(p); }
    void set_host_ptr(void *p, dim3 &s) { host_ptr = static_cast<T *>(p); set_size(s); }

    void memcpy_from_host(void *host_src) {
        set_host_ptr(host_src);
        memcpy_to_dev(host_src);
    }
    void memcpy_to_host(void *host_dst) { memcpy_from_dev(host_dst); }
    size_t elem_size() const { return sizeof(T); }
    T *dptr() const { return static_cast<T *>(device_ptr); }

  private:
    gpu_array(const gpu_array &) = delete;
    gpu_array &operator=(const gpu_array &) = delete;
    T *host_ptr = nullptr;  // never owned
};

#endif
