/*
 * kernel_manager.h -- kernel_manager / opencl_kernel of the reference
 * (common/inc/kernel_manager.h:7-21, common/inc/opencl_kernel.h:10-148).
 * There is nothing to build at run time: the kernels are sm_103a code in the
 * library.  kernel_manager becomes a name registry: Get_Kernel(name) returns
 * the launcher handle of a known kernel ("raycast" or "raycast.cl") and
 * throws std::runtime_error for an unknown one (the reference prints and
 * rethrows, kernel_manager.cpp:17-30).  The path argument is ignored.
 * add_kernel_arg(s)/execute are accepted for source compatibility; the
 * opencl_wrappers.h functions ignore the collected arguments.
 */
#ifndef TDE_3DEYE_KERNEL_MANAGER_H
#define TDE_3DEYE_KERNEL_MANAGER_H

#include <map>
#include <string>
#include <vector>

#include "gpu_array.h"

using std::string;
using std::vector;

class opencl_kernel {
  public:
    explicit opencl_kernel(const string &name, profiling_level profiling = DISABLE_PROFILING);
    ~opencl_kernel();
    const string get_name() const { return kernel_name; }
    void free_args();
    template <class T> void add_kernel_arg(T *) { ++num_args; }
    void add_kernel_arg(gpu_array_base *) { ++num_args; }
    template <class T> void add_kernel_args(T *arg) { add_kernel_arg(arg); }
    template <class T, class... Args> void add_kernel_args(T *arg, Args... args) {
        add_kernel_arg(arg);
        add_kernel_args(args...);
    }
    int num_kernel_args() const { return num_args; }
    void execute(const size_t *, const size_t *) {}
    void execute(const size_t *, bool = false) {}
    void execute(size_t, size_t, size_t, bool = false) {}

  private:
    string kernel_name;
    int num_args = 0;
};

class kernel_manager {
  public:
    kernel_manager(const string &path_to_kernels, vector<string> &names);
    ~kernel_manager();
    opencl_kernel *Get_Kernel(string &kernel_name);
    opencl_kernel *Get_Kernel(const char *kernel_name);
    string Get_Path() { return path; }

  private:
    std::map<string, opencl_kernel *> kernels;
    string path;
};

/* Names this library implements (strip a trailing ".cl" before lookup). */
bool tde_kernel_known(const string &name);

#endif
