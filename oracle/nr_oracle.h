/*
 * nr_oracle — CPU restatement of the reference's FIRE strain-and-relax path
 * (jmichelstl/network_relaxation, src/large_strain_relax.cu), in plain C.
 *
 * TEST INFRASTRUCTURE ONLY.  The test suite, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg use it to check results against; the product never links,
 * loads or calls it.
 *
 * Parity pin: tests/test_oracle_vs_reference.py checks this restatement
 * against the reference's own code compiled for the host
 * (oracle/build_ref.sh -> oracle/_ref/liblsr_ref.so) where the reference
 * checkout is present, and against tests/golden/ fixtures produced by that
 * build (tests/golden/make_golden.py) everywhere else.
 *
 * Arithmetic is "canonical": every operation, fused multiply-add and
 * summation order is fixed so the GPU kernels reproduce the same bits:
 *  - forces are summed per node in the reference's kernel order, all bonds in
 *    index order then all triples in index order (hinge, j, k roles), which is
 *    the reference's atomicAdd scatter (large_strain_relax.cu:386-469) with the
 *    atomics serialised in index order;
 *  - reductions over nodes / bonds / triples use or_canon_sum's fixed tree;
 *  - the bending angle uses or_atan2, a polynomial atan with fixed
 *    coefficients (no libm transcendental).
 * Build with -ffp-contract=off so the compiler adds no fused operations.
 */
#ifndef NR_ORACLE_H
#define NR_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Topology + positions as read from a .dat file (large_strain_relax.cu:42-114)
 * with triples from get_triples (:116-184). */
typedef struct {
    int n_points, n_edges, n_triples;
    double offset; /* x period ("width") */
    double miny, maxy;
    double *points;        /* 2*n_points, xy interleaved */
    int *edge_ij;          /* 2*n_edges */
    double *edge_l0;       /* n_edges */
    signed char *edge_wrap;/* n_edges: periodic image multiplier */
    int *tri_hjk;          /* 3*n_triples: hinge, j, k */
    signed char *tri_wrap; /* 2*n_triples: wrap of hinge->j, hinge->k */
} or_net;

/* Model seen by the force / energy / FIRE functions.  bond_k, tri_kb and
 * tri_phi0 are optional extensions (NULL = the reference's global ks, kb and
 * rest angle pi); tri_phi0 holds theta0 - pi per triple. */
typedef struct {
    int n_points, n_edges, n_triples;
    double width, ks, kb;
    const int *edge_ij;
    const double *edge_l0;
    const signed char *edge_wrap;
    const int *tri_hjk;
    const signed char *tri_wrap;
    const unsigned char *fcodes;
    const double *bond_k;
    const double *tri_kb;
    const double *tri_phi0;
    /* Gel coupling of network_mesh_relax.cu (all zero / NULL = none): FEM
     * triangles with their reference inverse matrices (get_inv_mats, :503-531,
     * 6 per element) and areas, pairs of duplicate mesh vertices, shear and
     * bulk moduli and the preferred dilation.  Active when bmod > 0 (:908, :952). */
    int n_elems, n_mpairs;
    double smod, bmod, gel_dilation;
    const int *elems;       /* 3*n_elems */
    const double *inv_mats; /* 6*n_elems */
    const double *areas;    /* n_elems */
    const int *mpairs;      /* 2*n_mpairs */
} or_model;

enum { OR_CRIT_RMS = 0, OR_CRIT_MAX = 1 };

typedef struct {
    double alpha0, falpha, dt_max, finc, fdec; /* fire_params[0..4] */
    int nmin;
    double mass, fcut;
    int max_steps;
    int criterion; /* OR_CRIT_RMS: |F|/sqrt(2N) < fcut (reference); OR_CRIT_MAX: max_i |F_i| < fcut */
} or_fire_params;

typedef struct {
    double rms_force, max_force, e_stretch, e_bend;
    int steps;
    int converged;
    double e_gel; /* report_data[3] of network_mesh_relax.cu's run_fire_md */
} or_report;

/* IO / topology (bit-exact restatements). */
int or_read_network(const char *path, or_net *net);           /* returns 1 iff the reference's read_network returns true */
void or_get_triples(or_net *net);                             /* fills tri_* (frees old) */
void or_free_net(or_net *net);
void or_fcodes(const or_net *net, const double *points, unsigned char *fcodes); /* :895-901 */
void or_affine_displace(int n_points, double *pos, double miny, double yrange, double xdisp, double ydisp);

/* Canonical math. */
double or_atan2(double y, double x);
double or_canon_sum(const double *terms, long n);

/* Physics. */
void or_forces(const or_model *m, const double *pos, double *forces);
void or_energies(const or_model *m, const double *pos, double *e_stretch, double *e_bend);
/* Virial {W_xx, W_yy, W_xy} of the stretch and bending forces (stress times
 * area); see nr_oracle.c. */
void or_virial(const or_model *m, const double *pos, double w[3]);
int or_fire(const or_model *m, double *pos, double *vel, double *forces, const or_fire_params *p, or_report *rep);

/* Strain protocol of do_relaxation_run (large_strain_relax.cu:917-999),
 * strain mode.  compr / shear = {min, max, inc} in strain units.  For every
 * relaxation it appends one record {curr_disp, max_comp, E_s, E_b, rms, maxF,
 * steps, is_shear} to records (capacity max_records) and, for shear steps,
 * copies the relaxed positions into shear_pos (2*n_points each, capacity
 * max_records).  Returns the number of records. */
int or_sweep(const or_model *m, double *pos, double miny, double yrange, const or_fire_params *p,
             const double compr[3], const double shear[3], double *records, int max_records,
             double *shear_pos);

/* Relaxes n independent models in parallel on n_threads host threads (one
 * network per thread at a time).  Each network uses or_fire. */
/* Post-relaxation analyses on reference positions pos0 and displacements
 * disp (2N each, xy interleaved); edges as (i, j) pairs with wrap codes.
 * strain_calc.cpp:96-120: per-bond (l_final - l_initial) / l_initial. */
void or_bond_strains(int n_edges, const int *edge_ij, const signed char *wrap, double width, const double *pos0,
                     const double *disp, double *strains);
/* axial_contribution.cpp:64-70 (unit bond vectors from pos0) and :176-190
 * (k/2 sum of the squared projections of the relative displacements); the
 * per-bond terms summed with or_canon_sum, then times k. */
double or_linear_axial_energy(int n_edges, const int *edge_ij, const signed char *wrap, double width, double k,
                              const double *pos0, const double *disp);
/* na_calc.cpp:308-327 (calc_na_val): mean over nodes of |u - u_affine|^2,
 * u_affine = (y - miny) (shear, axial); terms summed with or_canon_sum. */
double or_nonaffinity(int n_points, const double *pos0, const double *disp, double miny, double axial_strain,
                      double shear_strain);

void or_fire_batch(int n, const or_model *models, double **pos, const or_fire_params *params, or_report *reps,
                   int n_threads);

/* ---- network-mesh composites (network_mesh_relax.cu, nr_oracle_mesh.c) ---- */

/* read_network_mesh (network_mesh_relax.cu:72-230): net as or_read_network
 * fills it (offset, points, edges with l0, miny/maxy), plus facets (3F),
 * areas (F), duplicate pairs (2P) and minx/maxx.  Returns 1 iff the
 * reference's reader returns true. */
typedef struct {
    or_net net;
    int n_facets, n_areas, n_mpairs; /* facets and areas read (they differ only on failure) */
    int *facets;
    double *areas;
    int *mpairs;
    double minx, maxx;
} or_mesh;
int or_read_network_mesh(const char *path, or_mesh *mesh);
void or_free_mesh(or_mesh *mesh);
/* The duplicate-vertex search of read_network_mesh (:219-227) over points;
 * returns the number of pairs written to pairs (capacity 2*n_points ints). */
int or_mesh_pairs(int n_points, const double *points, double offset, double minx, int *pairs);
/* get_inv_mats (:503-531) from positions pos. */
void or_inv_mats(int n_elems, const double *pos, const int *elems, double *inv_mats);
/* dilate (:796-806) over the n_points nodes. */
void or_dilate(int n_points, double *pos, double minx, double miny, double factor);
/* gel_forces (:702-751) and duplicate_forces (:754-780) added to F, which
 * holds the network forces (or_forces calls this when m->bmod > 0). */
void or_gel_forces(const or_model *m, const double *pos, double *F);
/* gel_energy (:674-699) summed as cublasDasum does (absolute values), with
 * the canonical reduction. */
double or_gel_energy(const or_model *m, const double *pos);
/* The set-up of do_relaxation_run (:1256-1274): net_bmod = 2 E_s / area /
 * dilation^2 from the stretch energy of the dilated network (0 when
 * ks <= 0), and the preferred dilation dilation (bmod + net_bmod) / bmod. */
double or_preferred_dilation(double ks, double e_stretch_dilated, double area, double dilation, double bmod);
/* The compression then shear loops of network_mesh_relax.cu's
 * do_relaxation_run (:1276-1376), strain mode, on a prepared model (pos
 * dilated, m->gel_dilation the preferred dilation).  range = dilated height.
 * Records (9 doubles) {curr_disp, max_comp, E_s, E_b, E_gel, rms, max|F|,
 * steps, is_shear}; compression rows have curr_disp 0 and max_comp the
 * compression, as the reference's edata file prints them. */
int or_mesh_sweep(const or_model *m, double *pos, double miny, double range, const or_fire_params *p,
                  const double compr[3], const double shear[3], double *records, int max_records,
                  double *shear_pos);

/* ---- linear response (sparse_relax.cpp, nr_oracle_spr.c) ---- */

/* get_sparse_stiffness_mat (sparse_relax.cpp:434-480): upper-triangle
 * triplets in (row, col) order, values accumulated in the reference's call
 * order, |value| <= 1e-10 dropped.  rows/cols/vals may be NULL to count. */
long or_spr_stiffness(int n_points, const double *points, int n_edges, const int *edge_ij, const double *edge_l0,
                      const signed char *edge_wrap, double offset, double ks, double kb, double mu, int n_triples,
                      const int *tri_hjk, const signed char *tri_wrap, long *rows, long *cols, double *vals);
/* get_stretch_shear_energy / get_bending_energy (:49-96), sequential sums. */
void or_spr_energies(const double *points, int n_edges, const int *edge_ij, const double *edge_l0,
                     const signed char *edge_wrap, double offset, double ks, double kb, double mu, int n_triples,
                     const int *tri_hjk, const signed char *tri_wrap, const double *u, double *e_ss, double *e_bend);
/* affine_displacement (:528-538) or add_displacement (:513-525). */
void or_spr_bc(int n_points, const double *points, double miny, double maxy, double compression, double shear,
               int affine, const unsigned char *is_top, double *bc);

#ifdef __cplusplus
}
#endif
#endif
