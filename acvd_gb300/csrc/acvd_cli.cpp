// Native command-line drivers over the C ABI, with the reference programs' arguments:
//
//   acvd  file nvertices gradation [options]   (DiscreteRemeshing/Examples/ACVD.cxx)
//   acvdq file nvertices gradation [options]   (DiscreteRemeshing/Examples/ACVDQ.cxx)
//   anisotropic_remeshing_q file nvertices gradation [options]
//                                              (DiscreteRemeshing/Examples/AnisotropicRemeshingQ.cxx)
//
// Compiled three times from this file (ACVD_CLI_QEM selects ACVDQ, ACVD_CLI_ANISO
// AnisotropicRemeshingQ: the quadric-anisotropic metric, its curvature and principal
// directions computed on the original mesh, output <dir>Remeshing.ply).  The remeshing follows
// vtkDiscreteRemeshing::Remesh (DiscreteRemeshing/vtkDiscreteRemeshing.h:877-954):
// subdivision below SubsamplingThreshold x K, curvature of the original mesh when the
// gradation asks for it (interpolated through the subdivision), the reference's initial
// sampling, MinimizeEnergy, the ForceManifold loop, the coarse mesh (centroids stored as
// floats, dual triangles), FixMeshBoundaries; then ACVD's quadric post-placement
// (ACVD.cxx:217-291) or ACVDQ's PLY output (ACVDQ.cxx:368-376).  ACVDQ's fixed
// vertices (-fv ids, -ft faces; ACVDQ.cxx:246-280, 327-363) become the first clusters,
// anchored at those vertices.  Options that need parts this build does not have stop
// with an error; keys the program does not know are ignored, as the reference's are.
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <utility>
#include <vector>

#include "../../include/acvd_gpu.h"

namespace {

#if defined(ACVD_CLI_QEM)
const char* kProg = "ACVDQ";
const int kMetric = ACVD_METRIC_QEM;
#elif defined(ACVD_CLI_ANISO)
const char* kProg = "AnisotropicRemeshingQ";
const int kMetric = ACVD_METRIC_QUADRIC_ANISOTROPIC;
#else
const char* kProg = "ACVD";
const int kMetric = ACVD_METRIC_ISOTROPIC;
#endif

struct Mesh {
    std::vector<double> xyz;
    std::vector<int32_t> tri;
    std::vector<int32_t> row, col, ev;
    int64_t nv() const { return (int64_t)xyz.size() / 3; }
    int64_t nf() const { return (int64_t)tri.size() / 3; }
    int64_t ne() const { return (int64_t)ev.size() / 2; }
};

[[noreturn]] void die(const std::string& msg) {
    std::fprintf(stderr, "%s: %s\n", kProg, msg.c_str());
    std::exit(1);
}

void check(acvd_ctx* ctx, int code, const char* what) {
    if (code == ACVD_OK) return;
    die(std::string(what) + ": " + (ctx ? acvd_last_error(ctx) : acvd_io_last_error()));
}

void topology(Mesh& m) {
    int64_t ne = 0;
    check(nullptr, acvd_build_topology(m.nv(), m.nf(), m.tri.data(), nullptr, nullptr, nullptr, &ne),
          "acvd_build_topology");
    m.row.resize(m.nv() + 1);
    m.col.resize(2 * ne);
    m.ev.resize(2 * ne);
    check(nullptr, acvd_build_topology(m.nv(), m.nf(), m.tri.data(), m.row.data(), m.col.data(), m.ev.data(), &ne),
          "acvd_build_topology");
}

void set_mesh(acvd_ctx* ctx, const Mesh& m) {
    check(ctx, acvd_set_mesh(ctx, m.nv(), m.xyz.data(), m.nf(), m.tri.data(), m.row.data(), m.col.data(), m.ne(),
                             m.ev.data()),
          "acvd_set_mesh");
}

// integers read one after the other until one does not parse (`input >> id`)
std::vector<int32_t> read_ids(const char* path) {
    std::vector<int32_t> ids;
    std::ifstream in(path);
    int id;
    while (in >> id) ids.push_back(id);
    return ids;
}

void write_mesh(const std::string& path, const std::vector<double>& xyz, const std::vector<int32_t>& tri) {
    if (acvd_write_mesh(path.c_str(), xyz.data(), (int64_t)xyz.size() / 3, tri.data(), (int64_t)tri.size() / 3))
        die("writing " + path + ": " + acvd_io_last_error());
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 4) {
        std::printf("Usage : %s file nvertices gradation [options]\n"
                    "nvertices is the desired number of vertices\n"
                    "gradation defines the influence of local curvature (0=uniform meshing)\n"
                    "options: -b 0/1 boundary fixing, -m 0/1 manifold output, -s threshold subsampling, "
                    "-o directory, -of file, -q level, -d 0\n",
                    kProg);
        return 0;
    }
    const char* file = argv[1];
    int k = std::atoi(argv[2]);
    const double gradation = std::atof(argv[3]);
    int boundary_fixing = 0, force_manifold = 0, threshold = 10;
#if defined(ACVD_CLI_QEM) || defined(ACVD_CLI_ANISO)
    int level = 3;          // the metric's QuadricsOptimizationLevel
#else
    int level = 1;          // ACVD's post-placement eigenvalues
#endif
    std::string outdir, outfile = "simplification.ply";
    bool have_outdir = false;
    // custom density (vtkDiscreteRemeshing.h:603-640, defaults :1203-1206)
    std::string density_file;
    double density_max = 1.0, density_min = 0.1, density_factor = 0.001;
    // -l, -fv, -ft act on the mesh in the order given (the reference's argument loop)
    std::vector<std::pair<std::string, std::string>> mesh_ops;
    for (int a = 4; a < argc; a += 2) {
        if (a + 1 >= argc) die(std::string("option ") + argv[a] + " without a value");
        const std::string key = argv[a];
        const char* value = argv[a + 1];
        if (key == "-b") boundary_fixing = std::atoi(value);
#ifndef ACVD_CLI_ANISO
        else if (key == "-m") force_manifold = std::atoi(value);
#endif
        else if (key == "-s") threshold = std::atoi(value);
        else if (key == "-o") { outdir = value; have_outdir = true; }
        else if (key == "-of") outfile = value;
        else if (key == "-q") level = std::atoi(value);
        else if (key == "-np" || key == "-p") {}   // the threaded CPU engine's threads / pooling
        else if (key == "-d") {
            if (std::atoi(value) != 0) die("display needs a graphics stack; only -d 0 is available");
        } else if (key == "-w") {
            die("option " + key + " needs a part this build does not have");
        } else if (key == "-l") {
            if (!(std::atof(value) > 0.0)) die("-l needs a positive ratio");
            mesh_ops.emplace_back(key, value);
        }
#ifndef ACVD_CLI_ANISO
        else if (key == "-cd") density_file = value;
        else if (key == "-cmax") density_max = std::atof(value);
        else if (key == "-cmin") density_min = std::atof(value);
        else if (key == "-cf") density_factor = std::atof(value);
#endif
#ifdef ACVD_CLI_QEM
        else if (key == "-fv" || key == "-ft") {
            mesh_ops.emplace_back(key, value);
        }
#endif
    }
    if (k <= 0) die("nvertices must be positive");

    Mesh m;
    {
        double* xyz = nullptr;
        int32_t* tri = nullptr;
        int64_t nv = 0, nf = 0;
        check(nullptr, acvd_read_mesh(file, &xyz, &nv, &tri, &nf), "reading the input mesh");
        m.xyz.assign(xyz, xyz + 3 * nv);
        m.tri.assign(tri, tri + 3 * nf);
        acvd_free(xyz);
        acvd_free(tri);
    }
    topology(m);
    std::printf("load : %s\nMesh with %lld vertices, %lld faces, %lld edges\n", file, (long long)m.nv(),
                (long long)m.nf(), (long long)m.ne());
    // -l splits long edges (vtkSurface::SplitLongEdges); fixed vertices: -fv lists vertex
    // ids, -ft face ids whose vertices are fixed; the last of -fv / -ft wins
    std::vector<int32_t> fixed;
    bool has_fixed = false;
    for (const auto& op : mesh_ops) {
        if (op.first == "-l") {
            const double ratio = std::atof(op.second.c_str());
            std::printf("Splitting edges longer than %g times the average edge length\n", ratio);
            double* xyz = nullptr;
            int32_t* tri = nullptr;
            int64_t nv = 0, nf = 0;
            check(nullptr, acvd_split_long_edges(m.nv(), m.xyz.data(), m.nf(), m.tri.data(), ratio, &xyz, &nv, &tri, &nf),
                  "acvd_split_long_edges");
            m.xyz.assign(xyz, xyz + 3 * nv);
            m.tri.assign(tri, tri + 3 * nf);
            acvd_free(xyz);
            acvd_free(tri);
            topology(m);
        } else if (op.first == "-fv") {
            fixed = read_ids(op.second.c_str());
            has_fixed = true;
        } else {
            const std::vector<int32_t> faces = read_ids(op.second.c_str());
            std::vector<char> mark(m.nv(), 0);
            for (int32_t f : faces) {
                if (f < 0 || f >= m.nf()) die("-ft: face id " + std::to_string(f) + " outside the mesh");
                for (int q = 0; q < 3; q++) mark[m.tri[3 * (int64_t)f + q]] = 1;
            }
            fixed.clear();
            for (int64_t v = 0; v < m.nv(); v++)
                if (mark[v]) fixed.push_back((int32_t)v);
            std::printf("Added %d constraints on triangles\n", (int)faces.size());
            has_fixed = true;
        }
    }
    const std::vector<double> input_xyz = has_fixed ? m.xyz : std::vector<double>();
    if (has_fixed) {
        for (int32_t v : fixed)
            if (v < 0 || v >= m.nv()) die("fixed vertex id " + std::to_string(v) + " outside the mesh");
        k += (int)fixed.size();   // SetNumberOfClusters(numberOfSamples + fixed vertices)
        std::printf("Read %d fixed Ids\n", (int)fixed.size());
    }

    acvd_opts opts;
    acvd_default_opts(&opts);
    acvd_ctx* ctx = acvd_create(&opts);
    if (!ctx) die("acvd_create: no usable CUDA device");

    // curvature of the original mesh when the metric's gradation asks for it (the
    // anisotropic metric always needs it, with the principal directions)
    std::vector<double> ind;
    std::vector<float> pd;
    const bool need_pd = kMetric == ACVD_METRIC_QUADRIC_ANISOTROPIC;
    const bool need_ind = gradation > 0.0 || need_pd;
    bool original_on_device = false;
    if (need_ind) {
        set_mesh(ctx, m);
        original_on_device = true;
        ind.resize(m.nv());
        if (need_pd) pd.resize(6 * (size_t)m.nv());
        if (!density_file.empty() && !need_pd)
            check(nullptr, acvd_density_indicator(density_file.c_str(), m.nv(), m.xyz.data(), density_max, density_min,
                                                  density_factor, ind.data()),
                  "the custom density");
        else
            check(ctx, acvd_compute_curvature(ctx, ind.data(), need_pd ? pd.data() : nullptr), "acvd_compute_curvature");
    }
    // CheckSubsamplingRatio: subdivide while the mesh has fewer than threshold x K vertices
    int levels = 0;
    while (m.nv() < (int64_t)threshold * k) {
        if (m.nf() == 0 || levels >= 99) die("the mesh cannot be subdivided to SubsamplingThreshold x K vertices");
        // the reference interpolates only the indicator through the subdivision, and its
        // anisotropic metric then reads principal directions past their end
        if (need_pd) die("the quadric-anisotropic metric needs SubsamplingThreshold x K input vertices");
        std::printf("Subdividing mesh\n");
        Mesh s;
        const int64_t nout = m.nv() + m.ne();
        s.xyz.resize(3 * nout);
        s.tri.resize(12 * m.nf());
        std::vector<int32_t> p1(m.ne()), p2(m.ne());
        std::vector<double> ind2(need_ind ? nout : 0);
        check(ctx, acvd_subdivide(ctx, m.nv(), m.xyz.data(), m.nf(), m.tri.data(), m.row.data(), m.col.data(),
                                  m.ne(), m.ev.data(), need_ind ? ind.data() : nullptr, s.xyz.data(), s.tri.data(),
                                  p1.data(), p2.data(), need_ind ? ind2.data() : nullptr),
              "acvd_subdivide");
        topology(s);
        m = std::move(s);
        ind = std::move(ind2);
        original_on_device = false;
        levels++;
    }
    if (!original_on_device) set_mesh(ctx, m);
    check(ctx, acvd_set_metric(ctx, kMetric, need_ind ? ind.data() : nullptr, need_pd ? pd.data() : nullptr, gradation),
          "acvd_set_metric");
#if defined(ACVD_CLI_QEM)
    check(ctx, acvd_set_quadrics_optimization_level(ctx, level), "acvd_set_quadrics_optimization_level");
    check(ctx, acvd_set_unconstrained_initialization(ctx, 1), "acvd_set_unconstrained_initialization");
#elif defined(ACVD_CLI_ANISO)
    check(ctx, acvd_set_quadrics_optimization_level(ctx, level), "acvd_set_quadrics_optimization_level");
#else
    check(ctx, acvd_set_quadrics_optimization_level(ctx, 3), "acvd_set_quadrics_optimization_level");
#endif
    // the reference's initial sampling, then MinimizeEnergy
    std::vector<double> weights(m.nv());
    check(nullptr, acvd_vertex_weights(kMetric, m.nv(), m.xyz.data(), m.nf(), m.tri.data(), nullptr, nullptr,
                                       nullptr, need_ind ? ind.data() : nullptr, gradation, weights.data()),
          "acvd_vertex_weights");
    std::vector<int32_t> labels(m.nv());
    check(nullptr, acvd_initial_sampling_fixed(m.nv(), m.row.data(), m.col.data(), weights.data(), k,
                                               (int32_t)fixed.size(), fixed.data(), labels.data()),
          "acvd_initial_sampling");
    check(ctx, acvd_set_labels(ctx, k, labels.data()), "acvd_set_labels");
    if (has_fixed) {
        check(ctx, acvd_set_fixed_clusters(ctx, (int32_t)fixed.size(), fixed.data()), "acvd_set_fixed_clusters");
        check(ctx, acvd_set_anchor_items(ctx, (int32_t)fixed.size(), fixed.data()), "acvd_set_anchor_items");
    }
    acvd_stats st;
    check(ctx, acvd_minimize(ctx, &st), "acvd_minimize");
    std::printf("The clustering took :%g seconds.\nNumber of loops:\t%d\n", st.device_ms / 1000.0, st.sweeps);
    int32_t kk = k;
    if (force_manifold) {
        int32_t issues = 0;
        for (int pass = 0;; pass++) {
            check(ctx, acvd_force_manifold_step(ctx, &issues, &kk), "acvd_force_manifold_step");
            if (issues == 0) break;
            if (pass >= 1000) die("ForceManifold: issues left after 1000 passes");
            std::printf("%d topology issues, restarting minimization\n", issues);
            check(ctx, acvd_minimize(ctx, &st), "acvd_minimize");
        }
    }
    // the coarse mesh: centroids (the first non-empty cluster's for an empty one), as floats
    std::vector<int32_t> sizes(kk);
    std::vector<double> cent(3 * (size_t)kk);
    double etot = 0.0;
    check(ctx, acvd_get_clusters(ctx, sizes.data(), nullptr, nullptr, nullptr, cent.data(), nullptr, &etot),
          "acvd_get_clusters");
    int valid = 0;
    for (int c = 0; c < kk; c++)
        if (sizes[c] > 0) { valid = c; break; }
    std::vector<double> out_xyz(3 * (size_t)kk);
    for (int c = 0; c < kk; c++)
        for (int q = 0; q < 3; q++) out_xyz[3 * c + q] = (double)(float)cent[3 * (sizes[c] ? c : valid) + q];
    int64_t nt = 0;
    check(ctx, acvd_get_dual_mesh(ctx, nullptr, &nt), "acvd_get_dual_mesh");
    std::vector<int32_t> out_tri(3 * nt);
    check(ctx, acvd_get_dual_mesh(ctx, out_tri.data(), &nt), "acvd_get_dual_mesh");
    if (boundary_fixing) {
        int64_t np = 0, nb = 0;
        check(ctx, acvd_fix_mesh_boundaries(ctx, nullptr, &np, nullptr, &nb), "acvd_fix_mesh_boundaries");
        std::vector<double> bp(3 * np);
        std::vector<int32_t> bt(3 * nb);
        check(ctx, acvd_fix_mesh_boundaries(ctx, bp.data(), &np, bt.data(), &nb), "acvd_fix_mesh_boundaries");
        out_xyz.insert(out_xyz.end(), bp.begin(), bp.end());
        out_tri.insert(out_tri.end(), bt.begin(), bt.end());
    }
    std::printf("Coarse mesh: %lld vertices, %lld faces\n", (long long)out_xyz.size() / 3, (long long)nt);
#if defined(ACVD_CLI_ANISO)
    // AnisotropicRemeshingQ.cxx:232-247: <dir>Remeshing.ply, binary PLY
    write_mesh(outdir + "Remeshing.ply", out_xyz, out_tri);
    (void)have_outdir;
    (void)level;
#elif defined(ACVD_CLI_QEM)
    // the fixed vertices are the first output vertices, in place (ACVDQ.cxx:341-363)
    if (has_fixed) {
        for (size_t i = 0; i < fixed.size(); i++)
            for (int q = 0; q < 3; q++)
                if (input_xyz[3 * (size_t)fixed[i] + q] != out_xyz[3 * i + q]) {
                    std::printf("Error, vertex %d has been lost\n", (int)fixed[i]);
                    acvd_destroy(ctx);
                    return 1;
                }
        std::printf("Constraints on vertices have been checked\n");
    }
    // ACVDQ writes PLY whatever the name says
    const std::string path = outdir + outfile;
    std::string low = path;
    for (char& ch : low) ch = (char)std::tolower((unsigned char)ch);
    // the writer picks the format from the name (".vtk" before ".ply")
    std::string tmp = path;
    if (low.find(".ply") == std::string::npos || low.find(".vtk") != std::string::npos) tmp = path + ".acvdq.ply";
    write_mesh(tmp, out_xyz, out_tri);
    if (tmp != path && std::rename(tmp.c_str(), path.c_str()) != 0) die("renaming " + tmp);
#else
    if (level != 0) {
        write_mesh(outdir + "smooth_" + outfile, out_xyz, out_tri);
        std::vector<double> placed(3 * (size_t)kk);
        check(ctx, acvd_post_placement(ctx, level, placed.data()), "acvd_post_placement");
        // the driver moves its NumberOfSamples vertices, stored as floats
        for (int64_t i = 0; i < 3 * (int64_t)k && i < (int64_t)placed.size(); i++) out_xyz[i] = (double)(float)placed[i];
        std::printf("After Quadrics Post-processing : %lld vertices\n", (long long)out_xyz.size() / 3);
    }
    write_mesh((have_outdir ? outdir + "/" : std::string()) + outfile, out_xyz, out_tri);
#endif
    acvd_destroy(ctx);
    return 0;
}
