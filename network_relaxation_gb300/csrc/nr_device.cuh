/*
 * Device-side layout of a network and the pieces every FIRE kernel shares:
 * the canonical reductions and the grid barrier with a wait budget.
 *
 * HBM layout of one network (all arrays 16-byte aligned):
 *   x, v, f        double2[N]   positions, velocities, forces (xy pairs; the
 *                               reference's d_pos layout)
 *   fcode          uint8[N]
 *   bond           int4[E]      {i, j, wrap, 0}
 *   bond_l0        double[E]    rest length
 *   bond_k         double[E]    optional per-bond stiffness
 *   tri            int4[T]      {hinge, j, k, (wrap_j & 255) | (wrap_k & 255) << 8}
 *   tri_kb, tri_phi0 double[T]  optional per-triple stiffness, rest offset
 *   bptr/bent      int[N+1]/int[2E]  incidence: (bond << 1) | role
 *   tptr/tent      int[N+1]/int[3T]  incidence: (triple << 2) | role
 *   part           double[4 * n_units]  reduction partials
 *   epart          double[9 * M]  energy pass tile partials, M = the largest
 *                                 tile count of bonds, triples, elements:
 *                                 bonds E, Wxx, Wyy, Wxy at q = 0..3,
 *                                 triples at 4..7, gel elements E at 8
 * Networks embedded in a gel (network_mesh_relax.cu) add
 *   elem           int4[F]      FEM triangle {v1, v2, v3, 0}
 *   elem_inv       double[6F]   reference inverse matrix (get_inv_mats layout)
 *   elem_area      double[F]
 *   efrc           double4[3F]  per element and vertex the gel force terms
 *   eptr/eent      int[N+1]/int[3F] incidence: 3 * element + role
 *   partner        int[N]       duplicate vertex (-1: none)
 * Canonical reduction (identical to the oracle's or_canon_sum): items are
 * grouped in tiles of 256 (8 chunks of 32, one warp each); a chunk is reduced
 * by an xor butterfly (16, 8, 4, 2, 1), the 8 chunk sums of a tile by the tree
 * ((c0+c1)+(c2+c3))+((c4+c5)+(c6+c7)); tile sums are accumulated per lane
 * k = t mod 256 in increasing t and the 256 lane sums are reduced like a tile.
 */
#ifndef NR_DEVICE_CUH
#define NR_DEVICE_CUH

#include <cuda_runtime.h>
#include <stdint.h>

namespace nr {

constexpr int kTile = 256;
constexpr int kEpartLists = 9; /* lists of the energy pass partials (epart) */
constexpr int kChunk = 32;
constexpr unsigned kFull = 0xffffffffu;

struct FireParamsDev {
    double alpha0, falpha, dt_max, finc, fdec, mass, fcut;
    int nmin, max_steps, criterion, precision;
};

/* FIRE scalars of the mixed-precision path (fire_mixed.cu): the per-step
 * update runs in FP32, |F| and max|F| are the FP64 values certified at the
 * last anchor. */
struct MixScal {
    float dt, dtm, dtsq, alpha, na, a; /* na, a: mixing pending for the next pass A */
    float m2_anchor;                   /* max|F|^2 at the current anchor */
    float pad0;
    int since, step, mix_pending, zero_v, done, converged, status, n_anchor;
    double fmag, maxf;
};

/* Per-network FIRE state, written by one CTA after each reduction and read by
 * all CTAs of the network.  The barrier words sit on their own 128-byte line. */
struct __align__(128) FireState {
    double dt, dtm, dtsq, alpha;
    double mix_na, mix_a;
    double fmag, maxf, power, vmag;
    double e_stretch, e_bend;
    int mix_pending, zero_v, since, step;
    int done, converged, status, fp64_steps;
    MixScal mix;    /* mixed precision, multi-CTA teams */
    int anchor_now; /* mixed precision: the team re-anchors before the next pass */
    int yielded;    /* mixed precision: left at an anchor for a larger cluster (fire_dsm.cu) */
    double e_gel;   /* gel energy (networks embedded in a gel) */
    double vir[3];  /* virial {W_xx, W_yy, W_xy} of the stretch and bending forces */
    int pad[2];
    unsigned int bar_count, bar_gen, abort_flag, timeout_site;
    unsigned int pad2[28];
};

struct NetDev {
    int n, n_edges, n_triples, n_tiles;
    int use_bonds, use_triples, sub, n_units; /* sub = chunks per reduction unit (1,2,4,8) */
    double width, ks, kb, sqrt_dof;
    double area; /* width x (maxy - miny) at creation: stress = virial / area */
    double2 *x, *v, *f;
    const unsigned char *fcode;
    const int4 *bond;
    const double *bond_l0, *bond_k;
    const int4 *tri;
    const double *tri_kb, *tri_phi0;
    const int *bptr, *bent, *tptr, *tent;
    /* mixed precision (fire_mixed.cu): double-float displacement from the
     * anchor x (global copy, used when it does not fit shared memory), FP32
     * velocity and force, double-float anchor force; per bond and per triple
     * the FP32 anchor record and the FP32 force change of the current pass */
    float4 *u; /* {hi.x, hi.y, lo.x, lo.y}: one 16-byte load per node */
    float2 *vf, *ff, *fa_hi, *fa_lo;
    /* anchor records are indexed by bond / triple, or by item slot in the
     * distributed-shared-memory kernel */
    float4 *mb_data; /* anchor vector i -> j, {hi.x, hi.y, lo.x, lo.y} */
    float2 *mb_sk;   /* {|r_anchor| - l0, k} */
    float4 *mt_arms; /* anchor arms {a.x, a.y, b.x, b.y} (hinge -> j, hinge -> k) */
    float2 *mt_pk;   /* {theta_anchor - pi, kb} */
    float2 *bdf;     /* force change of the bond on node i */
    float4 *tdf;     /* force changes of the triple on j and k */
    double2 *bfrc;  /* FP64 path: force of every bond on its first endpoint */
    double4 *tfrc;  /* FP64 path: (F_j, F_k) of every triple */
    double *part;   /* 4 * n_units partial sums (P, V2, F2, maxF2) */
    double *epart;  /* kEpartLists * max(bond, triple, element tiles) energy partials */
    FireState *st;
    /* gel coupling (network_mesh_relax.cu), read only when use_gel; kept
     * behind one pointer so the descriptor the mixed-precision kernels
     * stage in shared memory stays small */
    int use_gel, n_elems;
    const struct NetGel *gel;
};

/* Gel of a network embedded in a gel: shear and bulk moduli, preferred
 * dilation (active when bmod > 0, network_mesh_relax.cu:908) and its FEM
 * triangles. */
struct NetGel {
    double smod, bmod, gdil;
    const int4 *elem;
    double *elem_inv;
    const double *elem_area;
    double4 *efrc; /* per element and vertex {x term 1, x term 2, y term 1, y term 2} */
    const int *eptr, *eent;
    const int *partner;
};

/* Layout of a network for the distributed-shared-memory cluster kernels
 * (fire_dsm.cu, fire_dsm64.cu).  Nodes are cut into 16 sub-blocks of bsub
 * consecutive nodes, bsub a multiple of 32; a cluster of C CTAs gives CTA r
 * the 16/C sub-blocks
 * [r 16/C, (r+1) 16/C), so one layout serves C = 1, 2, 4, 8, 16.  A bond
 * belongs to the sub-block of its node i, a triple to that of its hinge;
 * item slots list each sub-block's items in index order, so every CTA's
 * items are one contiguous slot range.
 *   node reference   sub-block << 16 | index within the sub-block
 *   bond entry       sub-block << 28 | slot << 1 | role
 *   triple entry     sub-block << 28 | slot << 2 | role
 * (entries parallel to NetDev bent / tent, in the same canonical order). */
constexpr int kDsmParts = 16;
struct NetDsm {
    int bsub;
    int bo[kDsmParts + 1], to[kDsmParts + 1]; /* first bond / triple slot of each sub-block */
    int be[kDsmParts + 1], te[kDsmParts + 1]; /* first bond / triple incidence entry of each sub-block */
    const int2 *bref;                         /* per bond slot: references of i, j */
    const int *bidx;                          /* per bond slot: bond index */
    const int4 *tref;                         /* per triple slot: references of h, j, k; triple index */
    const int *bent, *tent;
    /* gather records, per node slot: within each sub-block the nodes by
     * decreasing numbers of triple, then bond entries; {node | fcode << 28,
     * first bond entry, bond entries | triple entries << 16, first triple
     * entry} (entries: indices into bent / tent) */
    const int4 *grec;
};

/* Layout of one large network for the tiled mixed-precision kernel
 * (fire_tile.cu).  Nodes are binned into spatial tiles; a tile owns its
 * nodes and reaches a halo of other tiles' nodes through its items: every
 * bond with an endpoint and every triple with a node among its own nodes (an
 * item on a tile boundary belongs to every tile it touches and is evaluated
 * by each of them, identically).
 *
 * Node state lives in TILE ORDER: tile t's own nodes occupy positions
 * own_pos .. own_pos + no (own_pos a multiple of 16, the
 * range padded to whole 16s with unused positions), so a tile's own state is
 * contiguous; node_of_pos maps back to node ids (-1 for padding).  Own nodes
 * are ordered within their tile by their numbers of incidence entries.
 *
 * Everything read-only that a tile reads in a FIRE step is one contiguous,
 * 16-byte aligned record in `ro`, staged into shared memory by TMA bulk
 * copies (cp.async.bulk), segments in this order, each padded to 16 bytes:
 *   bref  nb x u32      local i | local j << 16
 *   mb    nb x float4   anchor vector i -> j {hi.x, hi.y, lo.x, lo.y}
 *   sk    nb x float2   {|r_anchor| - l0, k}
 *   tref  nt x uint2    {local h | local j << 16, local k}
 *   arms  nt x float4   anchor arms {a.x, a.y, b.x, b.y}
 *   pk    nt x float2   {theta_anchor - pi, kb}
 *   iptr  (no+1) x u16  incidence range of each own node (relative)
 *   ibe   no x u16      end of each own node's bond entries (its triple
 *                       entries follow up to the next iptr)
 *   inc   ni x u16      entries in the canonical order (bonds, then
 *                       triples): bond slot << 1 | role, triple 0x8000 |
 *                       slot << 2 | role
 *   fcode no x u8
 *   halo  nh x i32      tile-order position of each halo node
 * (local node k < no: own node k; no + h: halo node h).  The anchor records
 * (mb, sk, arms, pk) are rewritten there at every anchor.  The state
 * (u, v, F) is double buffered: a step reads one copy and writes the other,
 * so a tile can recompute its halo nodes' drift from the step's inputs while
 * their owners write theirs. */
struct TileDesc {
    long long ro_off; /* byte offset of the tile's record in ro */
    int own_pos, no, nh, nb, nt, ni;
    int bond_off, tri_off; /* first entry of the tile in bid / tid */
    int pad;
};
struct TileSegs {
    unsigned bref, mb, sk, tref, arms, pk, iptr, ibe, inc, fcode, halo, total; /* byte offsets in a tile record */
};
__host__ __device__ inline unsigned tile_pad16(unsigned b) { return (b + 15u) & ~15u; }
__host__ __device__ inline TileSegs tile_segs(int nb, int nt, int no, int ni, int nh) {
    TileSegs g;
    unsigned o = 0;
    g.bref = o;  o += tile_pad16(4u * nb);
    g.mb = o;    o += 16u * nb;
    g.sk = o;    o += tile_pad16(8u * nb);
    g.tref = o;  o += tile_pad16(8u * nt);
    g.arms = o;  o += 16u * nt;
    g.pk = o;    o += tile_pad16(8u * nt);
    g.iptr = o;  o += tile_pad16(2u * (no + 1));
    g.ibe = o;   o += tile_pad16(2u * no);
    g.inc = o;   o += tile_pad16(2u * ni);
    g.fcode = o; o += tile_pad16(1u * no);
    g.halo = o;  o += tile_pad16(4u * nh);
    g.total = o;
    return g;
}
struct NetTile {
    int n_tiles, n_pos;                  /* tiles; tile-order positions (with padding) */
    int max_nodes, max_bonds, max_tris;  /* per tile: own + halo nodes, bond items, triple items */
    int max_own;                         /* per tile: own nodes */
    unsigned max_ro;                     /* largest tile record, bytes */
    const TileDesc *desc;
    unsigned char *ro;                   /* tile records (anchor records rewritten in place) */
    const int *node_of_pos;              /* node id of each tile-order position (-1: padding) */
    const int *bid, *tid;                /* global bond / triple id of each tile item */
    float4 *u[2];                        /* double-buffered state, tile order: u {hi, lo}, */
    float4 *vf[2];                       /* and {v, F} */
    float4 *fa;                          /* double-float anchor force {hi, lo}, tile order */
    float *cpart;                        /* per CTA step totals (5 floats, two copies) */
    double *dpart;                       /* per CTA FP64 anchor totals (2 doubles each) */
    unsigned long long *bar;             /* grid barrier counter (monotonic) */
};

/* ----- reductions ----- */

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v = v + __shfl_xor_sync(kFull, v, off);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v = fmax(v, __shfl_xor_sync(kFull, v, off));
    return v;
}
__device__ __forceinline__ double tree2(const double *w) { return w[0] + w[1]; }
__device__ __forceinline__ double tree4(const double *w) { return (w[0] + w[1]) + (w[2] + w[3]); }
__device__ __forceinline__ double tree8(const double *w) {
    return ((w[0] + w[1]) + (w[2] + w[3])) + ((w[4] + w[5]) + (w[6] + w[7]));
}
/* Combines `sub` consecutive chunk sums with the lower levels of tree8. */
__device__ __forceinline__ double subtree(const double *w, int sub) {
    return sub == 8 ? tree8(w) : sub == 4 ? tree4(w) : sub == 2 ? tree2(w) : w[0];
}
/* Tile sum from the units of tile t (8/sub units, each a subtree of sub
 * chunks), finishing tree8's upper levels. */
__device__ __forceinline__ double tile_from_units(const double *p, int sub) {
    double u[8];
    const int upt = 8 / sub;
    for (int i = 0; i < upt; ++i) u[i] = __ldcg(p + i);
    if (sub == 8) return u[0];
    if (sub == 4) return u[0] + u[1];
    if (sub == 2) return (u[0] + u[1]) + (u[2] + u[3]);
    return ((u[0] + u[1]) + (u[2] + u[3])) + ((u[4] + u[5]) + (u[6] + u[7]));
}

/* Final stage of the canonical sum for the calling CTA: units[] holds
 * n_units unit partials (sub chunks each) of n_tiles tiles.  Every thread of
 * the CTA returns the same value.  smem: >= 8 doubles (one per warp of the
 * first 8 warps). */
__device__ inline double final_sum(const double *units, int n_tiles, int sub, double *smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int upt = 8 / sub; /* units per tile */
    for (int g = warp; g < 8; g += nwarps) {
        const int k = 32 * g + lane;
        double acc = 0.0;
        if (k < n_tiles) {
            acc = tile_from_units(units + (size_t)k * upt, sub);
            for (int t = k + kTile; t < n_tiles; t += kTile) acc = acc + tile_from_units(units + (size_t)t * upt, sub);
        }
        acc = warp_sum(acc);
        if (lane == 0) smem[g] = acc;
    }
    __syncthreads();
    const double r = tree8(smem);
    __syncthreads();
    return r;
}
/* Maximum of n_units partials; smem: one double per warp of the CTA. */
__device__ inline double final_max(const double *units, int n_units, double *smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    double m = 0.0;
    for (int u = threadIdx.x; u < n_units; u += blockDim.x) m = fmax(m, __ldcg(units + u));
    m = warp_max(m);
    if (lane == 0) smem[warp] = m;
    __syncthreads();
    double r = 0.0;
    for (int w = 0; w < nwarps; ++w) r = fmax(r, smem[w]);
    __syncthreads();
    return r;
}

/* ----- grid barrier with a wait budget ----- */

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

/* Arrive-and-wait across the `nblocks` CTAs sharing `st`.  The last CTA to
 * arrive returns is_last = true WITHOUT releasing the others: it must call
 * barrier_release() after finishing its serial work.  Returns false (and sets
 * st->abort_flag / st->status) when the wait exceeds budget_ns or another CTA
 * aborted; every thread of the CTA sees the same result. */
__device__ inline bool barrier_arrive(FireState *st, unsigned nblocks, unsigned long long budget_ns, bool &is_last,
                               unsigned site) {
    __shared__ int s_flag;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = &st->bar_gen;
        volatile unsigned *abort_flag = &st->abort_flag;
        int flag = -1;
        const unsigned g = *gen;
        if (!*abort_flag) {
            __threadfence();
            const unsigned prev = atomicAdd(&st->bar_count, 1u);
            if (prev == nblocks - 1) {
                atomicExch(&st->bar_count, 0u);
                __threadfence();
                flag = 1;
            } else {
                flag = 0;
                const unsigned long long t0 = global_ns();
                unsigned spins = 0;
                while (*gen == g) {
                    if (*abort_flag) {
                        flag = -1;
                        break;
                    }
                    if ((++spins & 63u) == 0 && global_ns() - t0 > budget_ns) {
                        atomicExch(&st->abort_flag, 1u);
                        atomicExch(&st->timeout_site, site);
                        flag = -1;
                        break;
                    }
                    __nanosleep(64);
                }
                __threadfence();
            }
        }
        s_flag = flag;
    }
    __syncthreads();
    const int flag = s_flag;
    __syncthreads();
    is_last = flag == 1;
    return flag >= 0;
}

__device__ __forceinline__ void barrier_release(FireState *st) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(&st->bar_gen, 1u);
    }
}

}  // namespace nr

#endif
