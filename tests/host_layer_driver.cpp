// A C++ caller of the host layer (rigid-ipc_gb300/host/rigid_ipc_gb300.hpp),
// built and run by tests/test_host_layer.py: it builds the reference-named
// classes from a scene file, runs one narrow-phase pass through them and
// writes the results, which the test compares with the Python binding's.
//
// File format (both ways): arrays one after the other, each an int64 count
// and the values (double or int32 as noted).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "rigid_ipc_gb300.hpp"

using namespace ipc::rigid::gb300;

template <class T> static std::vector<T> read_vec(FILE* f)
{
    int64_t n = 0;
    if (fread(&n, sizeof(n), 1, f) != 1 || n < 0) std::exit(3);
    std::vector<T> v((size_t)n);
    if (n && fread(v.data(), sizeof(T), (size_t)n, f) != (size_t)n) std::exit(3);
    return v;
}

template <class T> static void write_vec(FILE* f, const std::vector<T>& v)
{
    const int64_t n = (int64_t)v.size();
    fwrite(&n, sizeof(n), 1, f);
    if (n) fwrite(v.data(), sizeof(T), v.size(), f);
}

int main(int argc, char** argv)
{
    if (argc != 3) return 2;
    FILE* in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    SceneArrays s;
    s.rest_vertices = read_vec<double>(in);
    s.edges = read_vec<int32_t>(in);
    s.faces = read_vec<int32_t>(in);
    s.faces_to_edges = read_vec<int32_t>(in);
    s.body_vertex_start = read_vec<int32_t>(in);
    s.body_edge_start = read_vec<int32_t>(in);
    s.body_face_start = read_vec<int32_t>(in);
    s.group_ids = read_vec<int32_t>(in);
    s.body_types = read_vec<int32_t>(in);
    s.r_max = read_vec<double>(in);
    s.average_edge_length = read_vec<double>(in).at(0);
    const std::vector<double> x0 = read_vec<double>(in), x1 = read_vec<double>(in);
    const double dhat = read_vec<double>(in).at(0);
    std::fclose(in);
    try {
        DistanceBarrierRBProblem p(s);
        p.constraint().initial_barrier_activation_distance = dhat;
        const double toi = p.compute_earliest_toi(x0, x1);
        p.constraint().trajectory_type = TrajectoryType::PIECEWISE_LINEAR;
        const double toi_pl = p.compute_earliest_toi(x0, x1);
        const bool active = p.has_collisions(x0, x1);  // rigid CCD for either trajectory
        p.constraint().trajectory_type = TrajectoryType::RIGID;
        std::vector<double> g;
        BlockSparse H;
        const double e = p.compute_barrier_term(x0, g, H, true, true);
        Candidates c;
        detect_collision_candidates_rigid(p.assembler(), x0, x1, c);
        const double md = p.compute_min_distance(x0);
        const bool isect = p.detect_intersections(x0);
        FILE* out = std::fopen(argv[2], "wb");
        if (!out) return 2;
        write_vec(out, std::vector<double> { toi, e, md, isect ? 1.0 : 0.0, toi_pl, active ? 1.0 : 0.0 });
        write_vec(out, g);
        write_vec(out, H.row_ptr);
        write_vec(out, H.col);
        write_vec(out, H.val);
        write_vec(out, c.ee);
        write_vec(out, c.fv);
        std::fclose(out);
    } catch (const Error& err) {
        std::fprintf(stderr, "%s\n", err.what());
        return 1;
    }
    return 0;
}
