/*
 * Host stand-in for the CUDA runtime, used ONLY to compile the reference's
 * large_strain_relax.cu and network_mesh_relax.cu as plain C++ so that their
 * own host logic (readers, get_triples, run_fire_md, do_relaxation_run) and
 * their own kernel bodies run sequentially on the CPU.  This is test infrastructure for
 * pinning the oracle; nothing in the product links it.
 *
 * "Device" memory is host memory.  Every allocation is padded to 3x its size
 * plus 4 KiB, zero-filled: the reference's affine_displace is launched over
 * 2N threads for N nodes (large_strain_relax.cu:928, :970, guard `>` at :533)
 * and bending_energies guards with `>` (:502), so both touch entries past the
 * end of their arrays; network_mesh_relax.cu's dilate and affine_displace
 * are launched the same way (:1254, :1290).  On a GPU those writes land in whatever allocation
 * follows; here they land in the padding and are never read back.
 */
#ifndef NR_REFSHIM_CUDA_RUNTIME_H
#define NR_REFSHIM_CUDA_RUNTIME_H

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int x_ = 1, unsigned int y_ = 1, unsigned int z_ = 1) : x(x_), y(y_), z(z_) {}
};

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3
};

#define __global__
#define __device__
#define __host__

/* Thread coordinates seen by the emulated kernel bodies. */
extern dim3 blockIdx, blockDim, threadIdx, gridDim;

inline cudaError_t cudaMalloc(void **ptr, size_t size) {
    *ptr = calloc(3 * size + 4096, 1);
    return *ptr ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaFree(void *ptr) { free(ptr); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void *dst, const void *src, size_t n, cudaMemcpyKind) {
    if (n) memmove(dst, src, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemset(void *dst, int value, size_t n) {
    memset(dst, value, n);
    return cudaSuccess;
}
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline const char *cudaGetErrorString(cudaError_t) { return "host shim error"; }

/* Sequential emulation: every atomic is a plain read-modify-write. */
inline double atomicAdd(double *addr, double value) {
    double old = *addr;
    *addr = old + value;
    return old;
}
inline double rhypot(double x, double y) { return 1.0 / hypot(x, y); }

/* Runs a kernel body once per (block, thread) in row-major order.  The
 * reference's kernels use neither shared memory nor barriers, so this is an
 * exact sequential execution of the grid. */
template <class Kernel, class... Args>
void nr_ref_launch(dim3 grid, dim3 block, Kernel kernel, Args... args) {
    gridDim = grid;
    blockDim = block;
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx)
                for (unsigned tz = 0; tz < block.z; ++tz)
                    for (unsigned ty = 0; ty < block.y; ++ty)
                        for (unsigned tx = 0; tx < block.x; ++tx) {
                            blockIdx = dim3(bx, by, bz);
                            threadIdx = dim3(tx, ty, tz);
                            kernel(args...);
                        }
}

#endif
