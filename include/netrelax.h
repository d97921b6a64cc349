/*
 * netrelax.h — C ABI of the GB300 (sm_103a) implementation of the
 * quasi-static strain-and-relax loop for 2D elastic fiber networks
 * (FIRE minimisation of bond stretch + fiber bending).
 *
 * Reference: jmichelstl/network_relaxation, src/large_strain_relax.cu.
 * Every entry point names the reference interface it replaces.  Arrays keep
 * the reference's layouts: positions are 2*N doubles, xy interleaved; a bond
 * is (i, j, l0, wrap) with the periodic image of j at x + wrap*width; a
 * bending triple is (hinge, j, k, wrap_j, wrap_k); fcodes are 0 (clamped) or
 * 3 (free in x and y), bit 0 = x free, bit 1 = y free.
 *
 * Threading: no global mutable state except where stated; distinct handles
 * may be used from distinct host threads.  Device work is queued on the
 * stream passed in (a cudaStream_t, NULL = legacy default stream).
 *
 * The library needs a CUDA device for every entry point that touches device
 * memory; there is no CPU fallback.  Host-only entry points (network IO,
 * topology, generators, batch-file parsing) work without a GPU.
 */
#ifndef NETRELAX_H
#define NETRELAX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NR_ABI_VERSION 2

/* Replaces the reference's bool returns (true = ran, false = cudaMalloc
 * failed; large_strain_relax.cu:541-548, :596).  NR_OK and
 * NR_NOT_CONVERGED both correspond to the reference's `true`. */
typedef enum {
    NR_OK = 0,
    NR_NOT_CONVERGED = 1, /* step cap reached before the force criterion */
    NR_ERR_INVALID = -1,  /* bad argument */
    NR_ERR_IO = -2,       /* file could not be opened / written */
    NR_ERR_PARSE = -3,    /* malformed .dat or batch file */
    NR_ERR_CUDA = -4,     /* CUDA runtime error (message in nr_last_error) */
    NR_ERR_OOM = -5,      /* device allocation failed */
    NR_ERR_NONFINITE = -6,/* a force or position became NaN/inf */
    NR_ERR_TIMEOUT = -7,  /* a grid barrier exceeded its wait budget */
    NR_ERR_CAPACITY = -8  /* request exceeds a fixed capacity */
} nr_status;

const char *nr_status_string(int status);
/* Message of the last error raised on the calling host thread. */
const char *nr_last_error(void);
int nr_abi_version(void);

/* ------------------------------------------------------------------ */
/* Host-side networks                                                  */
/* ------------------------------------------------------------------ */

typedef struct nr_host_network nr_host_network;

typedef struct {
    int n_points, n_edges, n_triples;
    double offset;     /* x period ("width", the header's third field) */
    double miny, maxy; /* as computed by the reader (max starts at FLT_MIN) */
    int has_bond_k, has_tri_kb, has_tri_phi0;
} nr_host_info;

/* read_network (large_strain_relax.cu:42-114): same parsing rules, same
 * rest lengths l0 = sqrt(dx*dx + dy*dy), same error cases.  On NR_ERR_PARSE
 * the partially read network is still returned in *out (the reference keeps
 * going with whatever it read); the caller frees it.  Lines are parsed on
 * NR_IO_THREADS threads (default: all). */
int nr_read_network(const char *path, nr_host_network **out);

/* get_triples (large_strain_relax.cu:116-184): the collinear (antiparallel
 * to absolute tolerance 1e-10) bond pairs at each hinge, same set and order.
 * Replaces any triples already held. */
int nr_get_triples(nr_host_network *net);

/* Builds a network from arrays.  edge_l0 may be NULL: rest lengths are then
 * computed from the points exactly as read_network does. */
int nr_host_network_from_arrays(int n_points, const double *points, int n_edges, const int *edge_ij,
                                const double *edge_l0, const signed char *edge_wrap, double offset,
                                nr_host_network **out);
/* Extensions with no reference counterpart (the reference hard-wires one
 * ks, one kb and theta0 = pi): explicit triples with optional per-triple kb
 * and rest-angle offset phi0 = theta0 - pi, and per-bond stiffness. */
int nr_host_network_set_triples(nr_host_network *net, int n_triples, const int *tri_hjk, const signed char *tri_wrap,
                                const double *tri_kb, const double *tri_phi0);
int nr_host_network_set_bond_k(nr_host_network *net, const double *bond_k);
void nr_host_network_info(const nr_host_network *net, nr_host_info *info);
/* Copies out the arrays; any pointer may be NULL. */
void nr_host_network_arrays(const nr_host_network *net, double *points, int *edge_ij, double *edge_l0,
                            signed char *edge_wrap, int *tri_hjk, signed char *tri_wrap, double *bond_k,
                            double *tri_kb, double *tri_phi0);
/* fcodes (large_strain_relax.cu:895-901): 0 for y < miny+1e-10 or
 * y > maxy-1e-10, else 3. */
void nr_host_network_fcodes(const nr_host_network *net, unsigned char *fcodes);
/* Writes the .dat format read_network reads (%.17g, round-trips exactly). */
int nr_write_network(const nr_host_network *net, const char *path);
/* No reference counterpart: a binary copy of a host network (points, bonds,
 * rest lengths, triples, per-item constants, mesh; little-endian, FNV-1a
 * checksum) that loads without parsing and without get_triples.  A
 * truncated or corrupt file gives NR_ERR_PARSE. */
int nr_write_network_bin(const nr_host_network *net, const char *path);
int nr_read_network_bin(const char *path, nr_host_network **out);
/* report_displaced (large_strain_relax.cu:216-227): n_points xy pairs as
 * "%2.10le\t%2.10le\n" lines (host array), formatted in parallel. */
int nr_write_positions(const double *xy, int n_points, const char *path);
void nr_host_network_free(nr_host_network *net);

/* Renumbers the nodes for locality (no reference counterpart; the
 * reference keeps file order): NR_ORDER_MORTON sorts them along a Z-order
 * curve of their positions, NR_ORDER_RCM by reverse Cuthill-McKee on the
 * bond graph.  Points, bond / triple / facet / pair indices are remapped;
 * bonds and triples keep their order (so per-node force sums, rest lengths
 * and energies are unchanged, only permuted).  new_to_old (may be NULL)
 * receives n_points entries: the old index of each new node.  Useful before
 * nr_network_create / nr_batch_create for files numbered without locality:
 * the cluster kernel cuts networks into contiguous index ranges. */
enum { NR_ORDER_MORTON = 1, NR_ORDER_RCM = 2 };
int nr_host_network_reorder(nr_host_network *net, int method, int *new_to_old);

/* Synthetic inputs (no reference counterpart; the reference ships none).
 * Diluted triangular lattice, nx columns x ny rows, unit spacing, rows at
 * y = j*sqrt(3)/2, odd rows shifted by +0.5, x-periodic with period nx.
 * Node (i,j) owns its right, up-left and up-right bonds, each kept with
 * probability p (SplitMix64 stream from seed).  jitter > 0 moves every node
 * by U(-jitter, jitter) in x and y (top and bottom rows in x only, so they
 * stay clamped) before rest lengths are taken.  line_triples != 0 adds
 * bending triples along the three lattice directions wherever both
 * collinear bonds survive, with phi0 = rest angle - pi (exactly 0 force at
 * rest); line_triples == 0 leaves triples to nr_get_triples. */
int nr_gen_lattice(int nx, int ny, double p, double jitter, uint64_t seed, int line_triples,
                   nr_host_network **out);
/* Mikado network in the unit box: n_fibers straight fibers of length
 * fiber_len with uniform centres and angles, x-periodic, cut at y = 0 and
 * y = 1; every crossing becomes a node, segments between consecutive nodes
 * on a fiber become bonds with per-bond k = k0 / l0; dangling ends are
 * pruned repeatedly; consecutive segment pairs along a fiber become triples
 * with kb = kappa0 / mean(l0 of the two segments) and their rest angle. */
int nr_gen_mikado(int n_fibers, double fiber_len, double k0, double kappa0, uint64_t seed,
                  nr_host_network **out);

/* ------------------------------------------------------------------ */
/* FIRE parameters and reports                                         */
/* ------------------------------------------------------------------ */

enum { NR_CRIT_RMS = 0, NR_CRIT_MAX = 1 };
enum { NR_FP64 = 0, NR_MIXED = 1 };

typedef struct {
    /* fire_params[5] of run_fire_md (large_strain_relax.cu:610-614) */
    double alpha0, falpha, dt_max, finc, fdec;
    int nmin;
    double mass;
    double fcut;
    int max_steps;
    /* NR_CRIT_RMS: |F|/sqrt(2N) < fcut (large_strain_relax.cu:716);
     * NR_CRIT_MAX: max_i |F_i| < fcut. */
    int criterion;
    /* NR_FP64 (plain, bit-reproducible) or NR_MIXED (FP32 bulk with FP64
     * anchors, reductions and a final FP64 certification). */
    int precision;
} nr_fire_params;

/* report_data[3] of run_fire_md plus the step count and extras. */
typedef struct {
    double rms_force; /* report_data[0]: |F|/sqrt(2N) */
    double e_stretch; /* report_data[1] */
    double e_bend;    /* report_data[2] */
    double max_force; /* max_i |F_i| */
    int steps;        /* step_count */
    int status;       /* nr_status of this relaxation */
    int fp64_steps;   /* iterations taken in FP64 (mixed precision only) */
    int reserved;
    double e_gel;     /* report_data[3] of network_mesh_relax.cu's run_fire_md
                         (0 without a gel) */
    /* No reference counterpart (the reference reports no stress): the
     * stress of the stretch and bending forces at the returned positions,
     * sigma = W / A with the virial W = -sum_n r_n (x) F_n (per bond
     * W_ab = r_a f_b, r = r_j - r_i the minimum image, f the force on i; per
     * triple W_ab = -(a_a F_j,b + b_a F_k,b), a, b its arms) and A = the x
     * period times (maxy - miny) of the network as created.  stress_xy is
     * (1/A) dE/dgamma under the affine shear of affine_displace, stress_yy
     * the same for a y stretch: the secant shear modulus at strain gamma is
     * 2 (E - E_0) / (A gamma^2), the tangent one d stress_xy / d gamma.  The
     * FP64 path computes it with the canonical sums (bit-reproducible); the
     * gel of network_mesh_relax.cu adds no term. */
    double stress_xx, stress_yy, stress_xy;
} nr_report;

/* ------------------------------------------------------------------ */
/* Device-resident network                                             */
/* ------------------------------------------------------------------ */

typedef struct nr_network nr_network;

/* Uploads topology and positions, builds the per-node incidence lists
 * (copy_bond_data / copy_triple_data, large_strain_relax.cu:552-594, plus
 * the fcodes of :895-902).  Bonds are used when ks > 0 and triples when
 * kb > 0 (:629, :634).  Stream may be NULL. */
int nr_network_create(const nr_host_network *net, double ks, double kb, void *stream, nr_network **out);
int nr_network_destroy(nr_network *dnet);
int nr_network_n_points(const nr_network *dnet);
/* Position copies accept host (pageable or pinned) or device pointers. */
int nr_network_set_positions(nr_network *dnet, const double *host_xy, void *stream);
int nr_network_get_positions(const nr_network *dnet, double *host_xy, void *stream);
/* Device pointer to the 2*N positions (valid until destroy). */
double *nr_network_positions_device(nr_network *dnet);

/* affine_displace (large_strain_relax.cu:527-537) over the N nodes:
 * x += xdisp*(y-miny)/yrange; y += ydisp*(y-miny)/yrange, bit-exact. */
int nr_affine_displace(nr_network *dnet, double miny, double yrange, double xdisp, double ydisp, void *stream);

/* run_fire_md (large_strain_relax.cu:596-762) on a device network: v and F
 * reset, FIRE to the force criterion or max_steps, energies at the end.
 * Blocks until the report is on the host. */
int nr_relax(nr_network *dnet, const nr_fire_params *params, nr_report *report, void *stream);

/* Forces at the current positions (axial_forces + bending_forces,
 * large_strain_relax.cu:386-469), copied to host_f (2*N doubles). */
int nr_forces(nr_network *dnet, double *host_f, void *stream);
/* axial_energies + bending_energies summed (large_strain_relax.cu:472-523,
 * :743, :751). */
int nr_energies(nr_network *dnet, double *e_stretch, double *e_bend, void *stream);

/* No reference counterpart: stress {xx, yy, xy} (as nr_report's) and the
 * energies {E_stretch, E_bend} at the current positions, with the canonical
 * sums of nr_energies. */
int nr_stress(nr_network *dnet, double stress[3], double energies[2], void *stream);

/* One record per relaxation of the strain protocol (the values
 * do_relaxation_run prints, large_strain_relax.cu:942-954, :983-994). */
typedef struct {
    double curr_disp; /* shear displacement (compression rows: 0) */
    double max_comp;  /* compression displacement (compression rows: curr) */
    double e_stretch, e_bend, rms_force, max_force;
    int steps;
    int is_shear;
    int status;
    int fp64_steps;
    double e_gel; /* gel energy (nr_mesh_sweep; 0 without a gel) */
    double stress_xx, stress_yy, stress_xy; /* as in nr_report */
} nr_step_record;

/* The compression-then-shear loops of do_relaxation_run
 * (large_strain_relax.cu:917-999) in strain mode: displacements are
 * strain * yrange; each step applies the increment with affine_displace and
 * relaxes.  compr / shear = {min, max, inc}.  Writes up to max_records
 * records; shear_positions (host, may be NULL) receives the relaxed
 * positions of each shear step (2*N doubles per record). */
int nr_sweep(nr_network *dnet, double miny, double yrange, const nr_fire_params *params, const double compr[3],
             const double shear[3], nr_step_record *records, int max_records, int *n_records,
             double *shear_positions, void *stream);
/* nr_sweep with the whole protocol captured in one CUDA graph and launched
 * once: no host round trip between strain steps; the records and shear
 * positions are read after the last step (device buffers of 2*N doubles
 * per recorded shear step).  Same arguments and the same results, bit for
 * bit.  A mixed-precision network of up to 4096 nodes (relaxed in one CTA
 * under host control) is swept as nr_sweep does.  After a failed step the
 * network's positions are those after the last step. */
int nr_sweep_graph(nr_network *dnet, double miny, double yrange, const nr_fire_params *params,
                   const double compr[3], const double shear[3], nr_step_record *records, int max_records,
                   int *n_records, double *shear_positions, void *stream);

/* ------------------------------------------------------------------ */
/* Drop-in for run_fire_md with the reference's own device arrays      */
/* ------------------------------------------------------------------ */

/* bool run_fire_md(...) (large_strain_relax.cu:596): same arguments in the
 * same order and meaning, minus the dim3 launch shapes (the library picks
 * its own).  d_pos is updated in place; d_vel and d_forces receive the final
 * velocities and forces.  report_data = {RMS F, E_stretch, E_bend}.  Runs
 * the FP64 path with the RMS criterion.  Returns NR_OK / NR_NOT_CONVERGED
 * where the reference returns true. */
int nr_run_fire_md(int num_dof, int npairs, int ntriples, double width, double ks, double kb, double *d_pos,
                   double *d_vel, double *d_forces, const int *d_pair_list, const double *d_lengths,
                   const signed char *d_e_offsets, const int *d_triples, const signed char *d_t_offsets,
                   const unsigned char *d_fcodes, const double fire_params[5], double mass, double fcut,
                   int max_steps, int nmin, double report_data[3], int *step_count, void *stream);

/* ------------------------------------------------------------------ */
/* Networks embedded in a gel (src/network_mesh_relax.cu)              */
/* ------------------------------------------------------------------ */

/* A network-mesh composite is an nr_host_network with FEM triangles
 * ("facets"), their areas, and pairs of duplicate vertices on the mesh's
 * left and right edges whose forces are summed (the periodic seam of the
 * gel).  The gel's energy per triangle, with F the deformation gradient
 * from the reference state, is
 *   smod A (|F|^2 / det F - 2) / 2 + bmod A (det F - 1 - dilation)^2 / 2
 * (network_mesh_relax.cu:674-699); it acts when bmod > 0 (:908). */
typedef struct {
    int n_facets, n_areas, n_mesh_pairs; /* n_areas < n_facets only in a partially read file */
    double minx, maxx;                   /* as computed by the reader (max starts at FLT_MIN) */
} nr_mesh_info;

/* read_network_mesh (network_mesh_relax.cu:72-230): header "N E F offset",
 * N points, E edges "i j wrap", F facets "i j k", F areas (> 0), same
 * parsing rules and error cases; the duplicate pairs are found as the
 * reader finds them (:219-227: points within 1e-10 of minx paired with the
 * point at x + offset, same y, to 1e-10).  On NR_ERR_PARSE the partially
 * read network is still returned in *out. */
int nr_read_network_mesh(const char *path, nr_host_network **out);
/* Writes the format nr_read_network_mesh reads (%.17g, round-trips). */
int nr_write_network_mesh(const nr_host_network *net, const char *path);
/* Attaches facets / areas / duplicate pairs to a network; n_pairs < 0
 * finds the pairs from the points as the reader does. */
int nr_host_network_set_mesh(nr_host_network *net, int n_facets, const int *facets, const double *areas, int n_pairs,
                             const int *mesh_pairs);
/* Changes the x period.  do_relaxation_run scales it by sqrt(1 + dilation)
 * before get_triples and the relaxation (network_mesh_relax.cu:1141). */
int nr_host_network_set_offset(nr_host_network *net, double offset);
void nr_host_network_mesh_info(const nr_host_network *net, nr_mesh_info *info);
void nr_host_network_mesh_arrays(const nr_host_network *net, int *facets, double *areas, int *mesh_pairs);
/* Synthetic composite (no reference counterpart; the reference ships no
 * inputs): nx x ny unit grid plus a copy of column 0 at x = nx (paired with
 * column 0), every cell split along its up-right diagonal into two gel
 * triangles; network bonds right (periodic), up and up-right on columns
 * 0..nx-1, each kept with probability p (SplitMix64 from seed); jitter as in
 * nr_gen_lattice (column 0 and its copy move in y only). */
int nr_gen_lattice_mesh(int nx, int ny, double p, double jitter, uint64_t seed, nr_host_network **out);

/* Device networks created from a composite carry its triangles; their
 * reference inverse matrices are computed at nr_network_create from the
 * positions then (get_inv_mats, network_mesh_relax.cu:503-531, which the
 * reference runs before dilating).  The gel stays off until
 * nr_network_set_gel gives bmod > 0; gel-coupled networks relax on the FP64
 * path (nr_relax with NR_MIXED returns NR_ERR_INVALID). */
int nr_network_set_gel(nr_network *dnet, double smod, double bmod, double dilation);
/* get_inv_mats again, from the current positions. */
int nr_network_gel_inv_mats(nr_network *dnet, void *stream);
/* dilate (network_mesh_relax.cu:796-806): x = minx + factor (x - minx),
 * y likewise, over the N nodes. */
int nr_dilate(nr_network *dnet, double minx, double miny, double factor, void *stream);
/* {E_stretch, E_bend, E_gel}: axial_energies, bending_energies and
 * gel_energy summed (network_mesh_relax.cu:1030-1056; the gel term as
 * cublasDasum sums it, absolute values). */
int nr_mesh_energies(nr_network *dnet, double energies[3], void *stream);
/* The set-up of do_relaxation_run (network_mesh_relax.cu:1254-1274) on a
 * network created from the composite with its period already scaled:
 * dilate by sqrt(1 + dilation) about (minx, miny), net_bmod = 2 E_stretch /
 * area / dilation^2 (0 when ks <= 0), preferred dilation dilation (bmod +
 * net_bmod) / bmod (returned), and the gel set with it. */
int nr_mesh_prepare(nr_network *dnet, double smod, double bmod, double dilation, double area, double *pref_dilation,
                    void *stream);
/* The compression then shear loops of network_mesh_relax.cu's
 * do_relaxation_run (:1276-1376), strain mode (height = the dilated
 * height): the first displacement is min, later ones inc, and compression
 * lowers the height affine_displace uses as it goes.  Records as nr_sweep
 * (compression rows: curr_disp 0, max_comp the compression). */
int nr_mesh_sweep(nr_network *dnet, double miny, double height, const nr_fire_params *params, const double compr[3],
                  const double shear[3], nr_step_record *records, int max_records, int *n_records,
                  double *shear_positions, void *stream);

/* get_inv_mats (network_mesh_relax.cu:503) on the reference's device
 * arrays: d_facets 3 ints per triangle (valid node indices of d_pos, as
 * the reference's kernel assumes), d_inv_mats 6 doubles per triangle.
 * Asynchronous on stream. */
int nr_get_inv_mats(int n_facets, const double *d_pos, const int *d_facets, double *d_inv_mats, void *stream);
/* bool run_fire_md(...) of network_mesh_relax.cu:865: same arguments in the
 * same order and meaning, minus the dim3 launch shapes.  report_data =
 * {RMS F, E_stretch, E_bend, E_gel}.  Gel arrays are read only when
 * bmod > 0.  FP64 path, RMS criterion; NR_OK / NR_NOT_CONVERGED where the
 * reference returns true. */
int nr_mesh_run_fire_md(int num_dof, int npairs, int ntriples, int nelems, double width, double ks, double kb,
                        double smod, double bmod, double dilation, double *d_pos, double *d_vel, double *d_forces,
                        const int *d_pair_list, const double *d_lengths, const signed char *d_e_offsets,
                        const int *d_triples, const signed char *d_t_offsets, const int *d_elems,
                        const double *d_areas, const double *d_inv_mats, const int *d_mpairs, int n_mpairs,
                        const unsigned char *d_fcodes, const double fire_params[5], double mass, double fcut,
                        int max_steps, int nmin, double report_data[4], int *step_count, void *stream);

/* ------------------------------------------------------------------ */
/* Linear response (src/sparse_relax.cpp)                              */
/* ------------------------------------------------------------------ */

/* The reference's sp_relax does not run FIRE: it solves the harmonic
 * (linearised) problem K_ff u = -(P^T K) bc for the free nodes, K the
 * stiffness matrix of bond stretching (stiffness ks / l per bond,
 * sparse_relax.cpp:280-323), linearised bending of the collinear triples
 * (kb, :326-386) and background shear (mu, :390-429), P the projection that
 * removes the clamped top and bottom rows (:560-605), bc the applied
 * displacement field (affine, :528-538, or the top row only, :513-525). */
typedef struct nr_spr nr_spr;

typedef struct {
    int n_points, n_free_dofs, n_triples;
    long nnz_upper;    /* stored upper-triangle entries of K */
    long sell_entries; /* device storage of the reduced matrix (SELL-32, padded) */
    int iterations[2]; /* CG iterations of the last nr_spr_solve: unit compression, unit shear */
    double rel_residual[2];
    double minx, maxx, miny, maxy; /* read_network's ranges (max starts at FLT_MIN) */
} nr_spr_info_t;

/* One load point: what do_relaxation_run prints (SPR:820-870). */
typedef struct {
    double compression, shear; /* absolute displacements */
    double e_total, e_ss, e_bend; /* linearised energies (:49-96) */
    double residual;              /* ||rhs - K_ff u||_2, printed as "Residual RMS force" */
    int iterations, status;
} nr_spr_record;

/* get_sparse_stiffness_mat (sparse_relax.cpp:434-480) on the host: the
 * stored upper-triangle entries in (row, col) order, each the sum of its
 * contributions in the reference's call order, |value| <= 1e-10 dropped
 * (bit-identical to the reference).  Returns the count (arrays may be NULL
 * to count) or a negative nr_status.  No GPU needed. */
long nr_spr_assemble(const nr_host_network *net, double ks, double kb, double mu, long *rows, long *cols,
                     double *vals);
/* Assembles K (triples recomputed when kb > 0, as the reference does),
 * the reduced system and uploads it. */
int nr_spr_create(const nr_host_network *net, double ks, double kb, double mu, void *stream, nr_spr **out);
int nr_spr_destroy(nr_spr *spr);
void nr_spr_info(const nr_spr *spr, nr_spr_info_t *info);
/* Solves the unit compression and unit shear loads of one loading mode
 * (affine != 0: affine_displacement, else add_displacement) together by
 * Jacobi-preconditioned CG to ||r|| <= tol ||b|| (the reference's SPQR
 * solve, :793; on a singular system the minimum-norm solution, which is
 * what its -n null-space removal intends).  NR_NOT_CONVERGED when
 * max_iter is reached. */
int nr_spr_solve(nr_spr *spr, int affine, double tol, int max_iter, void *stream);
/* One load point from the unit solutions (linearity): u_final = bc + P u
 * (:812-813), residual of this point's own system, energies.  u_final
 * (2N doubles, host or device, may be NULL) receives the full
 * displacement field (the .disp file's values). */
int nr_spr_point(nr_spr *spr, double compression, double shear, nr_spr_record *rec, double *u_final, void *stream);

/* sp_relax's batch file (sparse_relax.cpp:931-1037): base [tag] / ks kb mu
 * / compression min max inc / shear min max inc. */
typedef struct {
    char base[1024];
    char tag[256];
    double ks, kb, mu;
    double compr[3], shear[3];
} nr_spr_spec;
int nr_parse_spr_batch_file(const char *path, nr_spr_spec *spec);
/* do_relaxation_run (sparse_relax.cpp:676-870) on one .dat file with the
 * reference's outputs (log with "Residual RMS force", energy file, .disp
 * files; empty names skip them).  strain_mode (-s): compression scaled by
 * the height, shear by the width (:728-737); affine (default; -z clears
 * it); itemize (-i): separate stretch+shear and bending columns. */
int nr_spr_do_relaxation_run(const char *dat_name, const char *log_name, const char *disp_base, const char *e_name,
                             const nr_spr_spec *spec, int strain_mode, int affine, int itemize);
/* run_relaxation_batch (:1042-1093): increments of ranges narrower than
 * 1e-10 become 1e12 (one value). */
int nr_spr_relaxation_batch(const char *batch_file, int strain_mode, int affine, int itemize);
/* The sp_relax command line (:1165-1232): -b batch [-s] [-z] [-i] [-n] [-g]
 * (-n and -g accepted: CG already gives the null-space-free solution, and
 * the solve always runs on the GPU). */
int nr_sp_relax_main(int argc, char **argv);

/* ------------------------------------------------------------------ */
/* Post-relaxation analyses                                            */
/* ------------------------------------------------------------------ */

/* The computations of the reference's analysis programs, on the GPU, for a
 * network given by its reference positions pos0 (2N doubles, xy) and a
 * displacement field disp (2N doubles), bonds as in nr_run_fire_md
 * (pair_list 2E ints, e_offsets E wrap codes, width = x period).  Arrays
 * may be host or device memory; the calls return when the results are
 * written.  Their scratch (device copies of host arrays, partial sums)
 * comes from a stream-ordered memory pool the library keeps per device,
 * which holds the largest scratch needed so far for the life of the
 * process.  Totals use the library's fixed summation tree (reproducible;
 * the reference sums sequentially, so they agree to rounding).
 *
 * strain_calc.cpp:96-120 (get_strains): strains[b] = (l_final - l_initial)
 * / l_initial, l_final from pos0 + disp. */
int nr_bond_strains(int n_points, int npairs, double width, const double *pos0, const double *disp,
                    const int *pair_list, const signed char *e_offsets, double *strains, void *stream);
/* axial_contribution.cpp:64-70, 176-190: *energy = k/2 sum_b ((u_j - u_i)
 * . r_hat_b)^2 with r_hat_b the unit bond vector in pos0. */
int nr_linear_axial_energy(int n_points, int npairs, double width, double k, const double *pos0,
                           const double *disp, const int *pair_list, const signed char *e_offsets, double *energy,
                           void *stream);
/* na_calc.cpp:308-327 (calc_na_val): *na = mean over nodes of
 * |u - u_affine|^2, u_affine = (y - miny) (shear_strain, axial_strain),
 * y from pos0. */
int nr_nonaffinity(int n_points, const double *pos0, const double *disp, double miny, double axial_strain,
                   double shear_strain, double *na, void *stream);

/* ------------------------------------------------------------------ */
/* Energies without allocating                                         */
/* ------------------------------------------------------------------ */

/* No counterpart in the reference: its energy step cudaMallocs a per-bond
 * and a per-triple array for every call (large_strain_relax.cu:738-758).
 *
 * Stretch and bend energies of a network held in the reference's device
 * layout (the arrays nr_run_fire_md takes; wrap codes as signed chars), with
 * the canonical FP64 sums of nr_energies (bit-identical results), for
 * callers that cannot allocate device memory: a host framework that hands
 * out all device memory from its own pool and forbids other allocations, or
 * a loop that must not pay for cudaMalloc / cudaFree, which can synchronize
 * the whole device.  It allocates nothing.  Its only scratch, the per-tile
 * partial sums, is a fixed array in the library's device memory: 2 x
 * NR_NOALLOC_MAX_ITEMS / 256 doubles (256 KiB), held on every GPU that
 * loads the library until the process exits.
 *
 * d_energies: device pointer to 2 doubles; receives {E_stretch, E_bend}
 * (a term is 0 when its stiffness is not positive).  npairs or ntriples
 * above NR_NOALLOC_MAX_ITEMS is rejected with NR_ERR_CAPACITY and a message
 * in nr_last_error.  A node index outside [0, n_points) makes the energy
 * NaN.  The first call on each device looks up the scratch array's device
 * address (this can load the library's device code): make that first call
 * before any stream capture.  The address is looked up again on every call,
 * so the entry point stays valid after cudaDeviceReset.  Every call uses the
 * same scratch array, so calls that overlap on the GPU (other streams or
 * host threads) race: issue all calls on one stream, or order calls on
 * different streams with events.  `stream` NULL (0) is the legacy default
 * stream, which orders the call after, and before, the work of every
 * blocking stream of the device; pass a framework's own stream (or
 * cudaStreamPerThread) to keep the call in that stream's order instead.
 * Nothing in the array needs clearing between calls.  Asynchronous on
 * `stream`. */
#define NR_NOALLOC_MAX_ITEMS 4194304
int nr_energies_noalloc(int n_points, int npairs, int ntriples, double width, double ks, double kb,
                        const double *d_pos, const int *d_pair_list, const double *d_lengths,
                        const signed char *d_e_offsets, const int *d_triples, const signed char *d_t_offsets,
                        double *d_energies, void *stream);

/* ------------------------------------------------------------------ */
/* Launch policy and the per-GPU tuning table                          */
/* ------------------------------------------------------------------ */

/* No reference counterpart (the reference's only launch knob is the block
 * shape, -x/-y, large_strain_relax.cu:1053-1090).  Each launch choice made
 * per size class -- kernel variant, CTAs per network, tile size, thresholds
 * between kernels, threads per CTA, escalation -- reads a named knob: the
 * environment variable of that name if set, else the loaded tuning table,
 * else the built-in default.  The table is loaded on first use from
 * NR_TUNING_FILE, else from tuning/<device name>.txt beside the library
 * (written by the autotuner, network_relaxation_gb300/autotune.py, from
 * measurements on that GPU).  Lines are "NAME value"; '#' starts a comment.
 * nr_tuning_load replaces the table (returns the entry count, NR_ERR_IO or
 * NR_ERR_PARSE); nr_tuning_value returns a knob's numeric value as the
 * library sees it (NaN when unset); nr_tuning_source names the table in use
 * ("" for none; the string stays valid for the life of the process, as
 * does every table loaded, so a load on one thread never invalidates what
 * another thread read). */
int nr_tuning_load(const char *path);
double nr_tuning_value(const char *name);
const char *nr_tuning_source(void);

/* No reference counterpart: the launch plan the library picks for this
 * network and precision (NR_FP64 / NR_MIXED) as text, e.g. "k_fire_dsm64
 * cluster=16" (NUL-terminated, truncated to cap). */
int nr_network_plan(nr_network *dnet, int precision, char *buf, size_t cap);

/* No reference counterpart; host only (no GPU needed): builds the spatial
 * tile layout that the tiled mixed-precision kernel would use for this
 * network with `ctas` CTAs and about `target_nodes` nodes per tile, and
 * checks every invariant the kernel relies on (each node owned by exactly
 * one tile, every local reference and incidence entry inside its tile,
 * bond entries before triple entries per node, 16-byte aligned records,
 * fcodes copied).  stats[0..5]: tiles, tile-order positions, largest tile
 * (own + halo nodes), largest record (bytes), halo nodes over all tiles,
 * violations found.  Returns NR_OK (violations counted in stats[5]) or
 * the builder's error (NR_ERR_CAPACITY, NR_ERR_INVALID). */
int nr_tile_layout_check(const nr_host_network *net, int ctas, int target_nodes, long long stats[6]);

/* No reference counterpart; host only: builds the sub-block layout of the
 * thread-block-cluster kernels for this network and checks it: every node
 * in exactly one gather record of its own sub-block, records ordered by
 * decreasing triple then bond entry counts, each record's entry ranges,
 * counts and fcode equal to the incidence lists, every bond and triple
 * slot owned by the sub-block of its first node / hinge, every resolved
 * incidence entry pointing at the item slot and role it came from.
 * stats[0..3]: sub-block size (nodes), sub-blocks in use, nodes,
 * violations found.  Returns NR_OK, or NR_ERR_CAPACITY when the network
 * exceeds the layout's encoding. */
int nr_dsm_layout_check(const nr_host_network *net, long long stats[4]);


/* ------------------------------------------------------------------ */
/* Batched relaxation of many independent networks in one launch       */
/* ------------------------------------------------------------------ */

typedef struct nr_batch nr_batch;

/* Uploads n networks into one set of device arrays.  ks[i], kb[i] per
 * network. */
int nr_batch_create(int n, const nr_host_network *const *nets, const double *ks, const double *kb, void *stream,
                    nr_batch **out);
int nr_batch_destroy(nr_batch *b);
int nr_batch_size(const nr_batch *b);
/* Kernel launches the last nr_batch_relax made on this batch (one, plus one
 * per escalation of long-running networks to larger thread-block clusters).
 * No counterpart in the reference, which relaxes one network at a time. */
int nr_batch_last_launches(const nr_batch *b);
/* No reference counterpart: the launch plan nr_batch_relax picks for this
 * batch and precision (kernel, CTAs per network, residency, single-CTA
 * networks, escalation), as nr_network_plan's text. */
int nr_batch_plan(nr_batch *b, int precision, char *buf, size_t cap);
int nr_batch_total_points(const nr_batch *b);
/* Positions of all networks, concatenated in network order (host or
 * device pointer). */
int nr_batch_set_positions(nr_batch *b, const double *host_xy, void *stream);
int nr_batch_get_positions(const nr_batch *b, double *host_xy, void *stream);
/* Device pointer to the concatenated positions. */
double *nr_batch_positions_device(nr_batch *b);
/* Per-network affine_displace with per-network miny, yrange, xdisp, ydisp
 * (host arrays of length n). */
int nr_batch_affine_displace(nr_batch *b, const double *miny, const double *yrange, const double *xdisp,
                             const double *ydisp, void *stream);
/* Relaxes every network (one persistent launch; each network's FIRE state
 * lives on the device; a network retires when it meets its criterion).
 * params: one nr_fire_params for all.  reports: n entries (host). */
int nr_batch_relax(nr_batch *b, const nr_fire_params *params, nr_report *reports, void *stream);
/* No reference counterpart (the reference sweeps one network at a time):
 * the compression-then-shear protocol of do_relaxation_run
 * (large_strain_relax.cu:924-999) in strain mode on every network of the
 * batch at once, each network's displacements scaled by its own
 * maxy - miny; per step one affine increment of every network and one
 * batched relaxation, warm-started from the previous step.  The steps are
 * counted in strain units (the same for every network).  graph != 0 records
 * the whole protocol as one CUDA graph and launches it once (escalation to
 * larger clusters is decided on the device); graph = 0 enqueues the same
 * work directly.  records: step-major, n_networks per step, up to max_steps
 * steps; *n_steps receives the protocol's step count.  The positions after
 * the sweep are the last step's. */
int nr_batch_sweep(nr_batch *b, const nr_fire_params *params, const double compr[3], const double shear[3],
                   nr_step_record *records, int max_steps, int *n_steps, int graph, void *stream);

/* ------------------------------------------------------------------ */
/* Driver, batch files and CLI                                         */
/* ------------------------------------------------------------------ */

typedef struct {
    char base[1024];
    char tag[256];
    double ks, kb;
    double fire_params[5];
    int nmin;
    double mass, fcut;
    int nmax;
    double compr[3], shear[3];
    /* 0: displacements are strain * (maxy - miny) (the reference's only
     * reachable mode); 1: absolute displacements (lsrelax -a). */
    int absolute;
    /* No reference counterpart: nonzero appends the shear and normal stress
     * (nr_report stress_xy, stress_yy) as two more columns to every _edata
     * line (lsrelax --stress); 0 keeps the reference's five columns. */
    int stress_columns;
} nr_batch_spec;

/* parse_batch_file (large_strain_relax.cu:297-383): six non-comment lines. */
int nr_parse_batch_file(const char *path, nr_batch_spec *spec);

/* get_file_lists (file_lists.cpp:80-138): the sorted .dat files matching
 * base*.dat and their _log.txt / _edata.txt / displacement-base names.
 * Returns the count, or a negative nr_status.  Names are written as
 * NUL-separated strings into buf (cap bytes); entry i occupies four
 * consecutive strings: dat, log, disp, edata. */
int nr_get_file_lists(const char *base, const char *ext, const char *tag, char *buf, size_t cap);

/* do_relaxation_run (large_strain_relax.cu:792-1010) on one network file:
 * reads it, builds triples when kb > 0, runs the protocol on the GPU and
 * writes the log, edata and NNN.pos files in the reference's formats.
 * precision / criterion select the path (the reference: NR_FP64, RMS). */
int nr_do_relaxation_run(const char *net_file, const char *log_name, const char *edata_name, const char *disp_base,
                         const nr_batch_spec *spec, int precision, int criterion);

/* relaxation_batch (large_strain_relax.cu:1016-1044). */
int nr_relaxation_batch(const char *batch_file, int precision, int criterion);

/* The lsrelax command line (large_strain_relax.cu:1047-1126):
 * -b batch [-x bx] [-y by] [-a] [-i], plus --precision fp64|mixed,
 * --criterion rms|max and --stress (two stress columns in _edata). */
int nr_lsrelax_main(int argc, char **argv);

/* nmrelax (network_mesh_relax.cu): the same driver for networks embedded in
 * a gel.  Its batch file's second line is "ks kb bmod smod dilation" (at
 * least three values; missing ones are 0), the network files are *.nmc. */
typedef struct {
    nr_batch_spec net;
    double bmod, smod, dilation;
} nr_mesh_batch_spec;
/* parse_batch_file (network_mesh_relax.cu:413-500). */
int nr_parse_mesh_batch_file(const char *path, nr_mesh_batch_spec *spec);
/* do_relaxation_run (network_mesh_relax.cu:1095-1390) on one .nmc file:
 * period scaled by sqrt(1 + dilation), triples, inverse matrices, dilation,
 * preferred dilation (printed), compression and shear loops with the gel,
 * and the log, edata (gel column and total) and NNN.pos files in the
 * reference's formats.  FP64 path. */
int nr_do_mesh_relaxation_run(const char *net_file, const char *log_name, const char *edata_name,
                              const char *disp_base, const nr_mesh_batch_spec *spec, int criterion);
/* relaxation_batch (network_mesh_relax.cu:1393-1421). */
int nr_mesh_relaxation_batch(const char *batch_file, int criterion);
/* The nmrelax command line (network_mesh_relax.cu:1424-1503), options as
 * nr_lsrelax_main (--precision is accepted; the gel runs in FP64). */
int nr_nmrelax_main(int argc, char **argv);

#ifdef __cplusplus
}
#endif
#endif
