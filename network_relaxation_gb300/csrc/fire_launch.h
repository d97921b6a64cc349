/* Host-side launchers of the FIRE kernels (defined in fire_fp64.cu,
 * fire_mixed.cu and fire_dsm.cu). */
#ifndef NR_FIRE_LAUNCH_H
#define NR_FIRE_LAUNCH_H

#include <cuda_runtime.h>

#include <vector>

#include "nr_device.cuh"

struct nr_host_network;

namespace nr {

/* A cooperative launch (all CTAs co-resident, as the grid barriers need),
 * expressed as a launch attribute so that stream capture records it as a
 * cooperative kernel node of a CUDA graph. */
inline cudaError_t launch_cooperative(const void *kernel, int blocks, int threads, void **args, size_t smem,
                                      cudaStream_t stream) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, kernel, args);
}

cudaError_t fp64_grid_max_blocks(int sub, bool gel, int *max_blocks);
/* stall: CTAs that never arrive, added to every grid barrier's count (0 in
 * normal use; the wait-budget test sets 1). */
cudaError_t launch_fp64_grid(const NetDev &d, const FireParamsDev &p, int blocks, unsigned long long budget_ns,
                             unsigned stall, cudaStream_t stream);
cudaError_t launch_energies(const NetDev &d, int blocks, cudaStream_t stream);
cudaError_t fp64_batch_max_blocks(int *max_blocks);
cudaError_t launch_fp64_batch(const NetDev *nets_dev, int n_nets, const FireParamsDev &p, int *queue_dev,
                              int blocks, cudaStream_t stream);
/* FP64 relaxation with one thread-block cluster of `cluster` CTAs (1..16)
 * per network, persistent over the queue (order_dev may be null): the
 * same bits as launch_fp64_grid. */
cudaError_t fp64_cluster_max_active(int cluster, bool gel, int *out);
cudaError_t launch_fp64_cluster(const NetDev *nets_dev, int n_nets, int cluster, bool gel, const FireParamsDev &p,
                                int *queue_dev, const int *order_dev, cudaStream_t stream);
/* FP64 relaxation with the step's state in distributed shared memory
 * (fire_dsm64.cu): one cluster of `cluster` CTAs per network over the
 * NetDsm layout, per-CTA maxima of nodes, bond slots and triple slots.  The
 * same bits as launch_fp64_grid. */
size_t dsm64_smem_bytes(int bmax, int emax, int tmax);
cudaError_t dsm64_max_active(int cluster, int bmax, int emax, int tmax, int *out);
cudaError_t launch_fp64_dsm(const NetDev *nets_dev, const NetDsm *dsm_dev, int n_nets, int cluster, int bmax,
                            int emax, int tmax, const FireParamsDev &p, int *queue_dev, const int *order_dev,
                            cudaStream_t stream);
cudaError_t launch_forces(const NetDev &d, cudaStream_t stream);
cudaError_t launch_affine(double2 *x, int n, double miny, double yrange, double xdisp, double ydisp,
                          cudaStream_t stream);
cudaError_t launch_affine_batch(const NetDev *nets_dev, const double4 *prm_dev, int n_nets, cudaStream_t stream);
/* get_inv_mats over n_elems triangles (vertex v of element e at
 * facets[stride * e + v]) and dilate over n nodes. */
cudaError_t launch_inv_mats(const double *pos, const int *facets, int stride, int n_elems, double *inv,
                            cudaStream_t stream);
cudaError_t launch_dilate(double2 *x, int n, double minx, double miny, double factor, cudaStream_t stream);

cudaError_t launch_mixed_batch(const NetDev *nets_dev, int n_nets, int max_nodes, const FireParamsDev &p,
                               int *queue_dev, const int *order_dev, cudaStream_t stream);

int mixed_cluster_size(int max_nodes);
cudaError_t launch_mixed_cluster(const NetDev *nets_dev, int n_nets, int cluster, const FireParamsDev &p,
                                 int *queue_dev, const int *order_dev, cudaStream_t stream);
size_t dsm_smem_bytes(int bmax, int emax, int tmax, int ebmax, int etmax, int resident);
size_t dsm_smem_limit();
/* One launch of the distributed-shared-memory kernel over n_nets networks
 * (order_dev[0..n_nets)); per-CTA maxima of nodes, bonds, triples and
 * incidence entries; resident: the CTAs keep their read-only slices in
 * shared memory too.  escalate > 0: once that fraction of the launched
 * clusters is idle, running networks stop at an anchor with their state
 * saved (FireState.yielded) for a relaunch on larger clusters.  queue_dev:
 * 2 ints (next slot, idle clusters). */
cudaError_t launch_mixed_dsm(const NetDev *nets_dev, const NetDsm *dsm_dev, int n_nets, int cluster, int bmax,
                             int emax, int tmax, int ebmax, int etmax, int resident, double escalate, int cap,
                             const FireParamsDev &p, int *queue_dev, const int *order_dev, cudaStream_t stream,
                             const int *n_dev = nullptr);
/* (launch_mixed_dsm: n_dev, when given, holds the launch's network count on
 * the device, at most n_nets.)  The yielded networks of a batch, compacted
 * on the device in index order: order_out and *count_out. */
cudaError_t launch_compact_yielded(const FireState *st, int n, int *order_out, int *count_out, cudaStream_t stream);
/* (launch_mixed_dsm: cap > 0 limits the number of clusters launched.)
 * Clusters of the given plan that fit the GPU at once. */
cudaError_t dsm_max_active(int cluster, int bmax, int emax, int tmax, int ebmax, int etmax, int resident, int *out);
/* Host arrays of a NetTile layout (fire_tile.cu). */
struct TileHost {
    int n_tiles = 0, n_pos = 0, max_nodes = 0, max_bonds = 0, max_tris = 0, max_own = 0;
    unsigned max_ro = 0;
    std::vector<TileDesc> desc;
    std::vector<unsigned char> ro;
    std::vector<int> node_of_pos, bid, tid;
};
struct Incidence;
/* The tiled mixed-precision kernel for one large network: layout, launch
 * width (co-resident CTAs for its shared memory) and launch. */
int build_tile_layout(const ::nr_host_network &h, const Incidence &inc, const unsigned char *fcodes, bool use_bonds,
                      bool use_triples, int ctas, int target_nodes, TileHost &out);
size_t tile_smem(const NetTile &tl);
int tile_grid_ctas(size_t smem, int threads);
cudaError_t launch_mixed_tile(const NetDev &d, const NetTile &tl, const FireParamsDev &p, int ctas, int threads,
                              unsigned long long budget_ns, cudaStream_t stream);
int mixed_grid_blocks(int n);
cudaError_t launch_mixed_grid(const NetDev &d, const FireParamsDev &p, int blocks, unsigned long long budget_ns,
                              cudaStream_t stream);

}  // namespace nr

#endif
