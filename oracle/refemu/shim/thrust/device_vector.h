/* Minimal stand-in for the one Thrust type the reference's GraphMeta.cuh
 * declares as members (thrust::device_ptr); its reductions and scans are run
 * by the emulation harness itself (test infrastructure only). */
#ifndef ASC_REFEMU_THRUST_H
#define ASC_REFEMU_THRUST_H
namespace thrust {
template <class T> struct device_ptr {
    T *p = nullptr;
    device_ptr() = default;
    explicit device_ptr(T *q) : p(q) {}
    T *get() const { return p; }
};
template <class T> struct plus { T operator()(const T &a, const T &b) const { return a + b; } };
}
#endif
