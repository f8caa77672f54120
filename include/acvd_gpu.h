/*
 * acvd_gpu.h -- C ABI of the GB300 (sm_103a) discrete Voronoi clustering engine.
 *
 * Drop-in for the energy-minimisation seam of ACVD's clustering path: the
 * reference calls vtkUniformClustering<Metric>::MinimizeEnergy()
 * (Common/vtkUniformClustering.h:264,725-830) from ProcessClustering()
 * (:655-714), itself called by vtkDiscreteRemeshing<Metric>::Remesh()
 * (DiscreteRemeshing/vtkDiscreteRemeshing.h:877-954).  These entry points take
 * the same inputs that seam reads -- the mesh, the per-vertex weights /
 * curvature data of the metric plugin, the initial clustering -- as plain host
 * arrays, run the minimisation on the GPU and hand back the clustering, the
 * cluster vertices and the dual (coarse) mesh.
 *
 * Conventions: ids are int32, vertex coordinates float64 xyz triples, triangles
 * int32 triples.  Labels lie in [0, K); K itself marks an unassigned item (the
 * reference's "null cluster", vtkUniformClustering.h:881-907).  The caller owns
 * every host buffer (copied in/out during the call); the context owns all device
 * memory.  A context is bound to one device and one CUDA stream and is not
 * thread-safe; separate contexts may run concurrently.  No function aborts:
 * each returns an ACVD_* status, with text from acvd_last_error().
 */
#ifndef ACVD_GPU_H
#define ACVD_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define ACVD_OK 0
#define ACVD_ERR_ARG 1          /* invalid argument or call order */
#define ACVD_ERR_CUDA 2         /* CUDA runtime error */
#define ACVD_ERR_ITER_LIMIT 3   /* an iteration cap was reached (MaxNumberOfLoops analogue) */
#define ACVD_ERR_DEVICE_CHECK 4 /* a device-side consistency check failed */
#define ACVD_ERR_UNSUPPORTED 5  /* input outside what this build handles */

/* metric plugins (DiscreteRemeshing/vtk*MetricForClustering.h) */
#define ACVD_METRIC_ISOTROPIC 0 /* vtkIsotropicMetricForClustering */
#define ACVD_METRIC_QEM 1       /* vtkQEMetricForClustering */
#define ACVD_METRIC_QUADRIC_ANISOTROPIC 2 /* vtkQuadricAnisotropicMetricForClustering */

typedef struct acvd_ctx acvd_ctx;

typedef struct acvd_opts {
    int device;              /* CUDA device ordinal */
    int use_graphs;          /* capture one sweep as a CUDA graph (1, default) */
    int max_loops;           /* sweep cap; reference MaxNumberOfLoops = 5,000,000 (:1407) */
    int max_convergences;    /* reference MaxNumberOfConvergences = 1e9 (:1406) */
    int kernel_timing;       /* record CUDA events around every evaluation kernel */
    int persistent;          /* run the sweeps between two convergence events in one cooperative
                                kernel with grid barriers (0, default; needs cooperative launch) */
} acvd_opts;

typedef struct acvd_stats {
    int sweeps;               /* colour sweeps run (the reference's NumberOfLoops analogue) */
    int convergences;         /* convergence events (reference :773-824) */
    int64_t moves;            /* committed moves */
    int64_t candidates;       /* proposed moves */
    int64_t boundary_items;   /* boundary items evaluated */
    int64_t targets;          /* (item, destination) energy evaluations */
    int64_t visited;          /* items visited by the evaluation kernels */
    int64_t slots;            /* ring slots read by the evaluation kernels */
    int disconnected;         /* clusters split at the last convergence */
    int unassigned;           /* items left unassigned after hole filling */
    double device_ms;         /* MinimizeEnergy on the device (CUDA events) */
    double eval_ms;           /* evaluation time: CUDA events per evaluation kernel (kernel_timing), or the
                                 device clock around the persistent kernel's evaluation phases */
    int eval_launches;        /* evaluation kernels timed */
    double energy;            /* global energy (FP64) of the final clustering */
    int64_t eval_bytes;       /* algorithmic bytes of all evaluation kernels (counted on device) */
    int64_t kernel_launches;  /* kernels launched by this call */
    int hit_loop_cap;         /* 1 if max_loops ended the minimisation (the reference just stops there too) */
    int64_t reverted;         /* commits undone because the pair's tracked energy did not decrease */
    int relaxed_sweeps;       /* sweeps run in relaxed (multi-move) mode */
    double sweep_kernel_ms;   /* persistent sweep kernels: CUDA-event time of all their launches */
    int sweep_kernel_launches; /* persistent sweep kernels launched (0 on the per-phase schedule) */
} acvd_stats;

/* Defaults: device 0, graphs on, per-phase kernels, the reference's loop caps. */
void acvd_default_opts(acvd_opts* opts);

acvd_ctx* acvd_create(const acvd_opts* opts);
void acvd_destroy(acvd_ctx* ctx);
const char* acvd_last_error(const acvd_ctx* ctx);

/*
 * Edge table and vertex rings in the reference's numbering
 * (vtkSurfaceBase::CreateFromPolyData, Common/vtkSurfaceBase.cxx:1407-1468,
 * AddEdge :1166-1221): faces are scanned in order and every new (v_j, v_j+1)
 * pair becomes the next edge; a vertex ring lists its edges in creation order.
 * Outputs: csr_row[nV+1], csr_col[2E] (ring neighbours), edge_v[2E].  Call with
 * NULL outputs first to get *n_edges.
 */
int acvd_build_topology(int64_t n_vertices, int64_t n_faces, const int32_t* tri, int32_t* csr_row,
                        int32_t* csr_col, int32_t* edge_v, int64_t* n_edges);

/*
 * Vertex weights of a metric plugin's BuildMetric, FP64 on the host:
 * dual area (Common/vtkSurface.cxx:1342-1359) times indicator^gradation, clamped
 * to [mean/ratio, mean*ratio] (ratio 1e5 isotropic / anisotropic, 1e4 QEM).
 * indicator may be NULL.  Used for the initial sampling below.
 */
int acvd_vertex_weights(int metric, int64_t n_vertices, const double* xyz, int64_t n_faces, const int32_t* tri,
                        const int32_t* csr_row, const int32_t* csr_col, const int32_t* edge_v,
                        const double* indicator, double gradation, double* weights);

/*
 * The reference's default initial sampling (InitSamples type 1 ->
 * ComputeInitialRandomSampling, Common/vtkUniformClustering.h:1178-1316):
 * std::mt19937 seeded 0 shuffles the items, regions grow breadth-first to the
 * average weight.  Writes labels[n_vertices] in [0, K] (K = unassigned).
 */
int acvd_initial_sampling(int64_t n_vertices, const int32_t* csr_row, const int32_t* csr_col,
                          const double* weights, int32_t k, int32_t* labels);

/*
 * The same with fixed vertices (SetFixedClusters, Common/vtkUniformClustering.h:134,
 * :1186-1190): vertex fixed_ids[c] starts in cluster c for c < n_fixed, the grown
 * regions take the labels n_fixed .. K-1 (acvd_initial_sampling is n_fixed = 0).  Where
 * every vertex is taken before the last region has started, the reference's loop
 * repeats forever (:1218-1232, the fixed vertices are never counted off); this
 * function goes on to split single vertices off the larger regions instead, as it
 * does when the regions outnumber what the growth reached.
 */
int acvd_initial_sampling_fixed(int64_t n_vertices, const int32_t* csr_row, const int32_t* csr_col,
                                const double* weights, int32_t k, int32_t n_fixed, const int32_t* fixed_ids,
                                int32_t* labels);

/*
 * vtkSurface::SplitLongEdges (Common/vtkSurface.cxx:444-603), host only: edges longer
 * than ratio x the mean edge length are split at their midpoints (stored as floats),
 * pass after pass until none is longer.  Vertices keep their ids, new ones are
 * appended in the reference's order, faces keep the reference's slots (a split face's
 * first part in its slot, the others appended); faces must be consistently oriented.
 * *out_xyz (3 out_nv doubles) and *out_tri (3 out_nf int32) are allocated with malloc;
 * release them with acvd_free.
 */
int acvd_split_long_edges(int64_t n_vertices, const double* xyz, int64_t n_faces, const int32_t* tri, double ratio,
                          double** out_xyz, int64_t* out_nv, int32_t** out_tri, int64_t* out_nf);

/*
 * Mesh upload (SetInput, vtkSurfaceClustering.h:179-211): coordinates, triangles
 * and the ring CSR / edge list from acvd_build_topology (or the caller's own
 * vtkSurface, exported in the same order).
 */
int acvd_set_mesh(acvd_ctx* ctx, int64_t n_vertices, const double* xyz, int64_t n_faces, const int32_t* tri,
                  const int32_t* csr_row, const int32_t* csr_col, int64_t n_edges, const int32_t* edge_v);

/*
 * Metric and its per-vertex inputs (Metric::BuildMetric, SetCurvatureInfo,
 * SetGradation): builds the float32 item records on the device.  indicator
 * (nV doubles) may be NULL when gradation is 0; principal_dirs (nV x 6 floats,
 * direction 1 then direction 2, scaled by sqrt|curvature|) is required by the
 * quadric-anisotropic metric only.
 */
int acvd_set_metric(acvd_ctx* ctx, int metric, const double* indicator, const float* principal_dirs,
                    double gradation);

/*
 * Batched meshes: n_mesh independent meshes packed into the arrays given to
 * acvd_set_mesh (vertex, face and edge ranges one after the other, ids global).
 * vertex_offsets[n_mesh+1] delimit each mesh's vertices; cluster_offsets[n_mesh+1]
 * each mesh's label range in [0, K).  Each mesh's weights are clamped against its
 * own mean, as when it is clustered alone; the minimisation runs all meshes in
 * the same sweeps (one CSR, one sweep graph).  Call after acvd_set_mesh and before
 * acvd_set_metric; n_mesh = 0 returns to a single mesh.  Batch of
 * DiscreteRemeshing/Examples/VolumeAnalysis.cxx:153-240, which runs one remesher
 * per mesh on CPU threads.
 */
int acvd_set_batch(acvd_ctx* ctx, int n_mesh, const int64_t* vertex_offsets, const int32_t* cluster_offsets);

/* Per-mesh global energies of a batch (energies[n_mesh]). */
int acvd_get_mesh_energies(acvd_ctx* ctx, double* energies);

/* Options of the reference API: SetQuadricsOptimizationLevel (default 3),
 * SetUnconstrainedInitialization (default 0). */
int acvd_set_quadrics_optimization_level(acvd_ctx* ctx, int level);
int acvd_set_unconstrained_initialization(acvd_ctx* ctx, int on);

/* SetNumberOfClusters + SetInitialClustering: K clusters, labels[nV] in [0, K].
 * Clears the frozen set below. */
int acvd_set_labels(acvd_ctx* ctx, int32_t k, const int32_t* labels);

/*
 * IsClusterFreezed (Common/vtkUniformClustering.h:329, tested at :912-915 and
 * :1049-1052): frozen[K] bytes, nonzero = frozen, or NULL for none.  The next
 * acvd_minimize moves no item out of a frozen cluster and none into it (an
 * unassigned item may still join one, as in the reference), and its early-
 * convergence base counts the items of the other clusters only (:733-736).
 * vtkDiscreteRemeshing's ForceManifold loop sets it before re-entering
 * MinimizeEnergy.  Call after acvd_set_labels.
 */
int acvd_set_frozen_clusters(acvd_ctx* ctx, const uint8_t* frozen);
/* The frozen set in force (K bytes, 1 = frozen; all 0 when none is set).  Reads what
 * the reference keeps in IsClusterFreezed; no entry of the reference corresponds. */
int acvd_get_frozen_clusters(acvd_ctx* ctx, uint8_t* frozen);

/*
 * SetFixedClusters (Common/vtkUniformClustering.h:134): cluster c < n_fixed is the
 * cluster of vertex vertex_ids[c].  CleanClustering keeps the component holding
 * that vertex, however small (:439-447); acvd_initial_sampling_fixed places the
 * vertices.  n_fixed = 0 clears the list.  Call after acvd_set_mesh; the list holds
 * until the next acvd_set_mesh, and n_fixed must not exceed K.
 */
int acvd_set_fixed_clusters(acvd_ctx* ctx, int32_t n_fixed, const int32_t* vertex_ids);

/*
 * Cluster::AnchorItem of the QEM metric (DiscreteRemeshing/vtkQEMetricForClustering.h:
 * 127-128; ACVDQ.cxx:333-334 sets it with the fixed vertices): cluster c < n is
 * anchored at vertex anchors[c] (-1: not anchored).  An anchored cluster's vertex
 * is its anchor (ComputeClusterCentroid :268-275), its energy W |p|^2 - 2 p.S
 * (:194-208), and a move of the anchor vertex out of it is never taken (the
 * reference prices it at 1e100, :194-200, :259).  ACVD_ERR_UNSUPPORTED for the other
 * metrics, whose clusters have no anchor.  Call after acvd_set_metric; the anchors
 * hold until the next acvd_set_mesh, across acvd_set_labels (clusters beyond n have
 * none).  n = 0 clears them.
 */
int acvd_set_anchor_items(acvd_ctx* ctx, int32_t n, const int32_t* anchors);

/*
 * CleanClustering (Common/vtkUniformClustering.h:406-549) on the current labels:
 * every cluster keeps its largest connected component (the earliest in vertex order
 * among equals; the one holding its fixed vertex, if any) and the items of the
 * others become unassigned (label K).  n_disconnected = the clusters that had
 * several components.  acvd_minimize runs it at each convergence; this entry runs it
 * alone.  Unlike the reference, the cluster whose first component starts at vertex 0
 * is cleaned as well (the reference's test VisitedCluster[Type] == 0, :463, skips it).
 */
int acvd_clean_clustering(acvd_ctx* ctx, int32_t* n_disconnected);

/*
 * MinimizeEnergy(): hole filling, statistics, colour sweeps until the
 * reference's stopping rule holds (0 moves in a sweep and 0 disconnected
 * clusters), with its early-convergence, unconstrained->constrained and
 * connectivity phases.  stats may be NULL.
 * Per-sweep log (the reference's SetWriteToGlobalEnergyLog, Common/vtkUniformClustering.h:
 * 1384-1395, as JSON lines): with the environment variable ACVD_SWEEP_LOG set to a file
 * path, every sweep appends {sweep, mode, moves, candidates, boundary_items, targets,
 * visited, screened, cached, reverted, energy (FP64 sum of the tracked cluster energies),
 * eval_ms (CUDA events around the evaluation kernels), eval_bytes, eval_gbs, sweep_ms,
 * constrained, connexity, convergences}, and every convergence event appends
 * {event, sweep, convergence, energy_tracked, energy_fp64 (a full FP64 recompute of the
 * same labels), rel_err}.  The sweeps then run from the host; the clustering is the same.
 */
int acvd_minimize(acvd_ctx* ctx, acvd_stats* stats);

/* Restores, on the device, the assignment last given to acvd_set_labels (no
 * host transfer), so that acvd_minimize can be repeated on resident inputs. */
int acvd_rewind(acvd_ctx* ctx);

/* GetClustering(): labels[nV]. */
int acvd_get_labels(acvd_ctx* ctx, int32_t* labels);

/*
 * Per-cluster results: sizes[K], FP64 accumulators S[3K] (sum w x), W[K]
 * (sum w), quadric[9K] (the reference's compact 9-coefficient quadric sum,
 * zeros for the isotropic metric), placed vertex centroid[3K] and energy[K].
 * Any output may be NULL.  Also returns the global energy in *energy_total.
 */
int acvd_get_clusters(acvd_ctx* ctx, int32_t* sizes, double* S, double* W, double* quadric, double* centroid,
                      double* energy, double* energy_total);

/* Edges whose endpoints carry different labels, in the reference's edge ids,
 * increasing.  Call with ids = NULL to get *count first. */
int acvd_get_boundary_edges(acvd_ctx* ctx, int32_t* ids, int64_t* count);

/*
 * The boundary edges of acvd_get_boundary_edges with no device allocation.  It
 * has no counterpart in the reference; it serves callers that hold the edge
 * table and the labels on the device already and must not allocate: a caller
 * that enqueues it inside its own stream-ordered loop, where the cudaFree of
 * acvd_get_boundary_edges would synchronise the whole device, or one whose
 * device memory is held by a caching allocator, where a cudaMalloc can fail.
 * Inputs are DEVICE arrays on the current device: d_edge_v[2 n_edges] (edge
 * endpoints, reference edge numbering), d_labels[nV]; outputs d_ids[n_edges]
 * (boundary edge ids, increasing) and d_count[1].  Enqueued on `stream` (a
 * cudaStream_t; NULL = the default stream) and returns without waiting.
 * Scratch is a fixed 256 KiB device array per device: no cudaMalloc, no
 * cudaFree.  The first call on a device looks that array's address up (set-up)
 * and keeps it for the process; make it before any stream capture.  After a
 * cudaDeviceReset of that device the kept address is stale: do not call this
 * entry point again in that process.  Calls on one device share the array, so calls
 * that overlap in time (other streams, other threads) race: serialise them.
 * n_edges above ACVD_NOALLOC_MAX_EDGES returns ACVD_ERR_UNSUPPORTED with
 * nothing enqueued.
 */
#define ACVD_NOALLOC_MAX_EDGES 67108864LL /* 2^26 edges */
int acvd_boundary_edges_noalloc(const int32_t* d_edge_v, int64_t n_edges, const int32_t* d_labels,
                                int32_t* d_ids, uint32_t* d_count, void* stream);

/*
 * Curvature of the mesh for vertex clustering, as vtkDiscreteRemeshing's
 * pre-processing computes it (DiscreteRemeshing/vtkDiscreteRemeshing.h:630-637 ->
 * Common/vtkCurvatureMeasure.cxx, polynomial fitting, vertices, 3-ring): per vertex
 * the indicator sqrt(k1^2 + k2^2) (indicator[nV]) and the two principal directions
 * scaled by sqrt|k|, the larger |k| first (principal_dirs[6 nV]); either output may
 * be NULL.  These are the arrays acvd_set_metric takes.  FP64 on the device.
 * Needs acvd_set_mesh.  A vertex whose 3-ring exceeds 192 faces returns
 * ACVD_ERR_UNSUPPORTED.
 */
int acvd_compute_curvature(acvd_ctx* ctx, double* indicator, float* principal_dirs);

/*
 * One level of midpoint subdivision, as vtkDiscreteRemeshing::CheckSubsamplingRatio
 * applies it while the input has fewer than SubsamplingThreshold x K vertices
 * (DiscreteRemeshing/vtkDiscreteRemeshing.h:841-875 -> vtkSurface::Subdivide,
 * Common/vtkSurface.cxx:605-677), with the parent interpolation of the vertex
 * indicator that the pre-processing applies afterwards (vtkDiscreteRemeshing.h:731-745).
 * Input: a mesh with its ring CSR and edge list from acvd_build_topology.
 * Outputs (host): out_xyz[3 (nV + nE)] -- the old points, then the midpoint of edge e
 * as vertex nV + e, each rounded to float as the reference's float vtkPoints stores
 * them; out_tri[12 nF] -- face f becomes faces 4f..4f+3 = (V1,V4,V6), (V4,V2,V5),
 * (V5,V3,V6), (V4,V5,V6), V4/V5/V6 the children of edges V1V2/V2V3/V3V1;
 * parent1/parent2[nE] -- the endpoints of edge e (VerticesParent1/2 of vertex nV + e);
 * out_indicator[nV + nE] -- indicator copied, then (ind[p1] + ind[p2]) * 0.5 (both
 * indicator and out_indicator NULL to skip).  The context gives the device and stream
 * only; its mesh is untouched.  A degenerate face (first two corners equal, which
 * vtkSurface treats as inactive) returns ACVD_ERR_UNSUPPORTED.
 */
int acvd_subdivide(acvd_ctx* ctx, int64_t n_vertices, const double* xyz, int64_t n_faces, const int32_t* tri,
                   const int32_t* csr_row, const int32_t* csr_col, int64_t n_edges, const int32_t* edge_v,
                   const double* indicator, double* out_xyz, int32_t* out_tri, int32_t* parent1, int32_t* parent2,
                   double* out_indicator);

/*
 * acvd_subdivide on device buffers (the same layouts, all in device memory of the
 * context's device), enqueued on the context's stream (acvd_stream): no allocation and
 * no synchronisation, for callers whose mesh is already resident.  No counterpart in the
 * reference, whose meshes live on the host.  d_work: at least
 * acvd_subdivide_work_bytes(n_edges) bytes, 16-byte aligned; after the stream reaches
 * this call, the uint32 at d_work + 8 n_edges bytes counts the faces that are
 * degenerate or have an edge missing from the ring CSR (their four output faces are
 * not written).  d_ind / d_out_ind may be NULL together.
 */
int64_t acvd_subdivide_work_bytes(int64_t n_edges);
int acvd_subdivide_device(acvd_ctx* ctx, int64_t n_vertices, const double* d_xyz, int64_t n_faces,
                          const int32_t* d_tri, const int32_t* d_row, const int32_t* d_col, int64_t n_edges,
                          const int32_t* d_edge_v, const double* d_ind, double* d_out_xyz, int32_t* d_out_tri,
                          int32_t* d_parent1, int32_t* d_parent2, double* d_out_ind, void* d_work);

/*
 * ACVD's quadric post-placement of the output vertices
 * (DiscreteRemeshing/Examples/ACVD.cxx:217-291, the ACVD driver's step after
 * Remesh()): per cluster, the unweighted plane quadrics of every face adjacent to
 * each of its items; each output vertex -- the metric's cluster centroid, the first
 * non-empty cluster's for an empty one -- moved by
 * vtkQuadricTools::ComputeRepresentativePoint with `level` singular values (ACVD's
 * default is 1).  FP64.  points: 3K doubles.
 */
int acvd_post_placement(acvd_ctx* ctx, int level, double* points);

/*
 * One pass of the ForceManifold loop of Remesh() (DiscreteRemeshing/vtkDiscreteRemeshing.h:
 * 937-950 -> DetectNonManifoldOutputVertices, :165-383) on the current clustering.  An
 * output vertex is checked on the coarse surface that BuildDelaunayTriangulation builds
 * under ForceManifold (the dual triangles plus an edge between every two adjacent
 * clusters, :1114-1132) with vtkSurfaceBase::IsVertexManifold's rule (at least two
 * edges, each with exactly two faces, one fan).  A non-empty cluster whose output
 * vertex fails and which holds no non-manifold input vertex is an issue: a new cluster
 * takes its first item (by vertex id; from a neighbouring cluster with more than one
 * item when it has a single one), and every cluster but the issues, their output
 * neighbours and the new ones is frozen.  On return *n_issues is the count (0: labels,
 * K and the frozen set unchanged -- the reference would leave every cluster frozen, which
 * only matters to a further MinimizeEnergy that Remesh() does not run); otherwise the context holds the new labels, K and frozen set, the
 * unconstrained first phase is off (the reference's metric stays constrained), and
 * acvd_minimize is the reference's re-entry into MinimizeEnergy.  *n_clusters is the
 * new K.  Loop while *n_issues > 0.
 */
int acvd_force_manifold_step(acvd_ctx* ctx, int32_t* n_issues, int32_t* n_clusters);

/*
 * FixMeshBoundaries (DiscreteRemeshing/vtkDiscreteRemeshing.h:426-579, Remesh()'s last
 * step when SetBoundaryFixing is on): the vertices and faces that close the coarse
 * mesh along the input's boundary, for the current clustering.  Pass 1: every input
 * boundary edge (one face) whose ends lie in two clusters gets a new vertex at its
 * midpoint (float-rounded, as the output's float vtkPoints stores it) and a face
 * (new, c1, c2).  Pass 2: every run of boundary edges inside one cluster joins that
 * cluster and the new vertices of the first two split edges it reaches.  Pass 3: a
 * boundary vertex next to two new vertices gets the face (its cluster, first, second)
 * -- only when the reference's GetNumberOfBoundaries (Common/vtkSurfaceBase.cxx:939-949,
 * which counts among the mesh's first `valence` edges rather than the vertex's) is
 * positive, as in the reference.  New vertices are numbered from K in order; faces are
 * listed in the order the reference adds them, corners as it passes them (its
 * vtkSurface may reorder corners to conquer an orientation; that is not replayed).
 * new_points: 3 x *n_new_points doubles, new_faces: 3 x *n_new_faces; on input the two
 * counts are the buffers' capacities.  Call with NULL buffers to get the counts.
 */
int acvd_fix_mesh_boundaries(acvd_ctx* ctx, double* new_points, int64_t* n_new_points, int32_t* new_faces,
                             int64_t* n_new_faces);

/*
 * Dual mesh (BuildDelaunayTriangulation, DiscreteRemeshing/vtkDiscreteRemeshing.h:1003-1152,
 * vertex clustering, without manifold repair): one triangle per input face whose
 * three labels are valid and distinct, in face order, duplicates (same label set)
 * dropped; corners in the face's vertex order.  Call with tris = NULL to get
 * *n_tris first.
 */
int acvd_get_dual_mesh(acvd_ctx* ctx, int32_t* tris, int64_t* n_tris);

/*
 * Adjoint for a fixed clustering (the labels last set or computed), FP64.
 * Inputs are DEVICE arrays: positions xyz[3 nV] and densities rho[nV] (the
 * per-vertex indicator, weight = area * rho^gradation; NULL for area weights).
 * Computes the metric energy sum_k E_k (host *energy), the per-cluster energies
 * cluster_energies[K] and the quadric-placed cluster vertices centroids[3K]
 * (device, either may be NULL), and, when grad_xyz is
 * given, the vector-Jacobian product of  g_energy * sum_k E_k + sum_k
 * g_centroids_k . c_k  with respect to xyz (grad_xyz[3 nV]) and rho
 * (grad_rho[nV], may be NULL).  The pseudo-inverse keeps the eigenvalues of its
 * forward evaluation (rank held fixed); clamped weights are constants.  Cluster
 * sums are recomputed on every call, nothing per item is stored.  Isotropic and
 * QEM metrics.
 */
int acvd_adjoint(acvd_ctx* ctx, const double* xyz, const double* rho, double gradation, double g_energy,
                 const double* g_centroids, double* energy, double* cluster_energies, double* centroids,
                 double* grad_xyz, double* grad_rho);

/*
 * acvd_adjoint ordered on the caller's CUDA stream (a cudaStream_t), with no host
 * synchronisation: the work waits on the device for what the caller enqueued on
 * `stream` before the call, and the caller's later work on `stream` waits for the
 * outputs.  The energy's cotangent d_g_energy and the energy d_energy are DEVICE
 * scalars (either may be NULL: cotangent 0, energy not returned).  This is what an
 * autograd function inside a training loop calls (acvd_gb300/csrc/adjoint_torch.cpp:
 * torch::autograd::Function on torch's current stream).  It has no counterpart in
 * the reference, whose clustering has no gradients.
 */
int acvd_adjoint_on_stream(acvd_ctx* ctx, void* stream, const double* xyz, const double* rho, double gradation,
                           const double* d_g_energy, const double* g_centroids, double* d_energy,
                           double* cluster_energies, double* centroids, double* grad_xyz, double* grad_rho);

/* The CUDA stream (cudaStream_t) the context launches on. */
void* acvd_stream(acvd_ctx* ctx);

/*
 * Failure detection without a fault: every device wait of this library (the grid
 * barrier of the persistent sweep kernel) gives up after a limited number of naps,
 * sets an error flag that the host reads, and returns, leaving the context usable.
 * This runs that barrier with one of two blocks never arriving and a limit of
 * max_spins naps of 64 ns (at most 2^24); *gave_up is 1 when the wait ran out as it
 * must.  A self-check with no counterpart in the reference.
 */
int acvd_check_wait_limit(acvd_ctx* ctx, int64_t max_spins, int32_t* gave_up);

/*
 * Triangle-mesh files, host only: the formats vtkSurface::CreateFromFile / WriteToFile
 * dispatch on by name (Common/vtkSurface.cxx:1958-2136; the lower-cased name contains
 * ".vtk", ".vtp", ".ply", ".off", ".obj" or ".stl", tested in the reference's order).  Read:
 * PLY (ascii / binary either endian), OFF, OBJ, STL (ascii / binary; identical corners
 * merged in order of first appearance, triangles left degenerate dropped), legacy VTK
 * POLYDATA (ascii / binary), VTK XML PolyData (ascii, inline base64 or appended data;
 * uncompressed or zlib; pieces concatenated).  Write: PLY (binary little endian, float
 * points), OFF, OBJ, STL (binary), legacy VTK (ascii), VTK XML (inline base64, float
 * points).  Only triangles: another polygon is ACVD_ERR_UNSUPPORTED, as are .wrl, triangle
 * strips and .vtp data under another compressor.  acvd_read_mesh allocates *xyz (3 nV
 * doubles) and *tri (3 nF int32) with malloc; release them with acvd_free.  The text of
 * the last failure of this thread is acvd_io_last_error().  acvd_free and
 * acvd_io_last_error have no counterpart in the reference (VTK owns its readers' memory
 * and reports through its error macros).
 */
int acvd_read_mesh(const char* path, double** xyz, int64_t* n_vertices, int32_t** tri, int64_t* n_faces);

/*
 * Custom density (vtkDiscreteRemeshing::SamplingPreProcessing with an InputDensityFile,
 * DiscreteRemeshing/vtkDiscreteRemeshing.h:603-640; the drivers' -cd / -cmax / -cmin /
 * -cf, defaults 1, 0.1, 0.001): the curvature indicator replaced, at each vertex, by
 * max(max_density - value * factor, min_density), value being the volume's voxel at the
 * cell holding the vertex (floor((x - origin) / spacing), the last cell at the upper
 * face; 0 outside the volume).  Host only.  The volume is a MetaImage file (.mhd with its
 * data file, or .mha; raw or zlib-compressed); MINC (.mnc) is ACVD_ERR_UNSUPPORTED.
 */
int acvd_density_indicator(const char* image_path, int64_t n_vertices, const double* xyz, double max_density,
                           double min_density, double factor, double* indicator);
int acvd_write_mesh(const char* path, const double* xyz, int64_t n_vertices, const int32_t* tri, int64_t n_faces);
void acvd_free(void* p);
const char* acvd_io_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* ACVD_GPU_H */
