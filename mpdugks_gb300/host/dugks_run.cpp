// dugks_run: the host-side solver driver around libdugks_gpu.so, the GPU
// counterpart of the reference's main() + DUGKS2DSolver()
// (Ark/Cpp/main.cpp:134, Ark/Cpp/DUGKS2DSolver.cpp:148-337).
//
//   dugks_run run <Case.ark> [--out DIR] [--precision P] [--steps N]
//                 [--mesh FILE.cas] [--checkpoint FILE] [--resume FILE]
//                 [--set key=value ...]
//       Reads the case from a Case.ark (the reference's OutputCase layout),
//       initialises it on the GPU, writes DIR/Case.ark and the FlowField at
//       step 0, then steps until End_Step (or --steps) or until the density
//       residual, evaluated every ResidualControl steps, falls below
//       RESIDUAL; FlowField files every writeFileControl steps and at the end
//       (DIR/global/, the reference's names and layout).  With --mesh the
//       grid comes from a .cas mesh file, as in the reference's
//       MeshConstruct, and the FlowField cells follow the mesh's cell order.
//       --checkpoint writes the whole GPU state (dugks_gpu_checkpoint) to FILE
//       at every FlowField output point and at the end; --resume restores
//       such a file after the initialisation and continues from its step.
//       The Allen-Cahn models also write the reference's line profiles into
//       DIR/Convergence/ (Ark/Cpp/DUGKS2DSolver.cpp:326-333,836-841): Diag and
//       MidX at every FlowField output point, Diag, MidX and MidY at the end
//       (Diag only when ny >= nx).  --l2 (the reference's
//       _OUTPUT_L2NORM_ERROR_FLIP, drop initialisations only) appends
//       AC_Drop_L2Norm at every residual point to
//       DIR/Convergence/L2_uvp_mu<Mu0>_Re<Re>_<mesh>.dat (Output_L2Norm,
//       Ark/Cpp/Output.cpp:239-256) and prints "L2_phi <value>" at the end.
//   dugks_run rewrite-ark <in> <out>        parse a Case.ark and write it back
//   dugks_run rewrite-flowfield <in> <out>  parse a FlowField file and write it back
//   dugks_run rewrite-profile <MidX|MidY|Diag> <nx> <ny> <in> <out>
//                                           parse a line-profile file and write it back
//   dugks_run mesh-info <FILE.cas>          nx ny y_walls, then the grid
//                                           position j*nx+i of every mesh cell
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/dugks_gpu.h"
#include "case_ark.hpp"
#include "flowfield.hpp"
#include "mesh_cas.hpp"
#include "profiles.hpp"

using namespace dugks_host;

namespace {

void check(dugks_handle_t *h, int rc, const char *what) {
    if (rc == DUGKS_OK) return;
    char buf[512] = {0};
    dugks_gpu_last_error(h, buf, sizeof(buf));
    throw std::runtime_error(std::string(what) + ": " + buf);
}

void make_dir(const std::string &d) {
    if (mkdir(d.c_str(), 0755) != 0) {
        struct stat st;
        if (stat(d.c_str(), &st) != 0 || !S_ISDIR(st.st_mode)) throw std::runtime_error("cannot create " + d);
    }
}

FlowField fields(dugks_handle_t *h, const RunConfig &c, const CartesianMap *mesh) {
    FlowField ff;
    ff.cells = (size_t)c.grid.nx * c.grid.ny;
    for (auto *v : {&ff.rho, &ff.u, &ff.v, &ff.p, &ff.T, &ff.phi, &ff.tau, &ff.fx, &ff.fy}) v->assign(ff.cells, 0.0);
    check(h, dugks_gpu_download(h, ff.rho.data(), ff.u.data(), ff.v.data(), ff.phi.data(), ff.p.data()), "download");
    check(h, dugks_gpu_get_field(h, DUGKS_F_TAU, ff.tau.data()), "tau");
    check(h, dugks_gpu_get_field(h, DUGKS_F_FX, ff.fx.data()), "Fx");
    check(h, dugks_gpu_get_field(h, DUGKS_F_FY, ff.fy.data()), "Fy");
    ff.T.assign(ff.cells, c.T0);  // isothermal models keep the reference temperature
    if (mesh)  // the reference writes cells in its CellArray order, the mesh file's
        for (auto *v : {&ff.rho, &ff.u, &ff.v, &ff.p, &ff.T, &ff.phi, &ff.tau, &ff.fx, &ff.fy})
            *v = to_mesh_order(*mesh, *v);
    return ff;
}

void output(dugks_handle_t *h, const RunConfig &c, const CartesianMap *mesh, const std::string &dir,
            int64_t step) {
    const std::string path =
        dir + "/global/" + flowfield_name(step, (double)step * c.dt, c.mach, c.mesh_type, c.nl, c.cfl);
    write_flowfield(path, fields(h, c, mesh));
}

bool allen_cahn(const RunConfig &c) {
    return c.cs.model == DUGKS_MODEL_AC || c.cs.model == DUGKS_MODEL_HCZ;
}

// the reference's line profiles at this step (Output_MidX / MidY / Diag)
void write_profiles(dugks_handle_t *h, const RunConfig &c, const std::string &dir, int64_t step, bool midy) {
    ProfileFields f;
    f.nx = c.grid.nx;
    f.ny = c.grid.ny;
    f.m_phi = c.cs.M_Phi;
    const size_t n = (size_t)f.nx * f.ny;
    for (auto *v : {&f.rho, &f.p, &f.tp, &f.u, &f.v}) v->assign(n, 0.0);
    check(h, dugks_gpu_download(h, f.rho.data(), f.u.data(), f.v.data(), nullptr, f.p.data()), "download");
    check(h, dugks_gpu_thermo_pressure(h, f.tp.data()), "thermodynamic pressure");
    const double ratio = c.cs.RhoL / c.cs.RhoV;
    auto put = [&](Profile k) {
        const std::string path = dir + "/Convergence/" + profile_name(k, c.mach, c.mesh_type, c.nl, c.cfl, ratio, step);
        std::FILE *o = std::fopen(path.c_str(), "wb");
        if (!o) throw std::runtime_error("cannot write " + path);
        const std::string text = format_profile(k, f);
        const size_t w = std::fwrite(text.data(), 1, text.size(), o);
        if (std::fclose(o) != 0 || w != text.size()) throw std::runtime_error("write failed: " + path);
    };
    if (f.ny >= f.nx) put(Profile::Diag);
    put(Profile::MidX);
    if (midy) put(Profile::MidY);
}

// one line t, L2(phi), L2_p = 0 (Output_L2Norm's layout, %.8e)
void append_l2(dugks_handle_t *h, const RunConfig &c, const CaseArk &ark, const std::string &dir, int64_t step) {
    double l2 = 0.0;
    check(h, dugks_gpu_drop_l2(h, &l2), "drop L2 norm");
    const std::string path = dir + "/Convergence/L2_uvp_mu" + ark.get("dynamic viscosity", "0.1") + "_Re" +
                             ark.get("Re", "0") + "_" + c.mesh_name + ".dat";
    std::FILE *o = std::fopen(path.c_str(), "ab");
    if (!o) throw std::runtime_error("cannot write " + path);
    std::fprintf(o, "%.8e    %.8e    %.8e\n", (double)step * c.dt, l2, 0.0);
    if (std::fclose(o) != 0) throw std::runtime_error("write failed: " + path);
}

// the whole GPU state to a file (written to FILE.tmp, then renamed)
void checkpoint_file(dugks_handle_t *h, const std::string &path) {
    size_t n = 0;
    check(h, dugks_gpu_checkpoint_bytes(h, &n), "checkpoint size");
    std::vector<char> buf(n);
    check(h, dugks_gpu_checkpoint(h, buf.data(), n), "checkpoint");
    const std::string tmp = path + ".tmp";
    std::FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + tmp);
    const size_t w = std::fwrite(buf.data(), 1, n, f);
    if (std::fclose(f) != 0 || w != n) throw std::runtime_error("write failed: " + tmp);
    if (std::rename(tmp.c_str(), path.c_str()) != 0) throw std::runtime_error("cannot rename " + tmp);
}

// restore a checkpoint file; returns its step
int64_t restore_file(dugks_handle_t *h, const std::string &path) {
    std::FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<char> buf;
    char chunk[1 << 16];
    size_t r;
    while ((r = std::fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + r);
    std::fclose(f);
    check(h, dugks_gpu_restore(h, buf.data(), buf.size()), "restore");
    int64_t steps = 0;
    check(h, dugks_gpu_step_count(h, &steps), "step count");
    return steps;
}

int run(int argc, char **argv) {
    if (argc < 3) throw std::runtime_error("run: missing Case.ark");
    CaseArk ark = read_case_ark(argv[2]);
    std::string out = "FlowField", mesh_file, ckpt_file, resume_file;
    int64_t steps_override = -1;
    bool l2 = false;
    for (int k = 3; k < argc; ++k) {
        const std::string a = argv[k];
        auto next = [&]() -> std::string {
            if (k + 1 >= argc) throw std::runtime_error(a + ": missing value");
            return argv[++k];
        };
        if (a == "--out") out = next();
        else if (a == "--precision") ark.set("precision", next());
        else if (a == "--steps") steps_override = std::atoll(next().c_str());
        else if (a == "--mesh") mesh_file = next();
        else if (a == "--checkpoint") ckpt_file = next();
        else if (a == "--resume") resume_file = next();
        else if (a == "--l2") l2 = true;
        else if (a == "--set") {
            const std::string kv = next();
            const size_t eq = kv.find('=');
            if (eq == std::string::npos) throw std::runtime_error("--set wants key=value");
            ark.set(kv.substr(0, eq), kv.substr(eq + 1));
        } else throw std::runtime_error("unknown option " + a);
    }
    RunConfig c = config_from_case_ark(ark);
    if (steps_override >= 0) c.end_step = steps_override;
    CartesianMap mesh;
    if (!mesh_file.empty()) {  // the grid is the mesh file's
        mesh = cartesian_map(read_cas(mesh_file));
        c.grid.nx = mesh.nx;
        c.grid.ny = mesh.ny;
        c.grid.y_walls = mesh.y_walls;
    }
    const CartesianMap *pm = mesh_file.empty() ? nullptr : &mesh;
    make_dir(out);
    make_dir(out + "/global");
    const bool ac = allen_cahn(c);
    if (ac) make_dir(out + "/Convergence");
    if (l2 && !(ac && (c.init_kind == 0 || c.init_kind == 1)))
        throw std::runtime_error("--l2 needs an Allen-Cahn case with a drop initialisation");
    write_case_ark(out + "/Case.ark", ark);

    dugks_handle_t *h = nullptr;
    int rc = dugks_gpu_create(&c.cs, &c.grid, &h);
    if (rc != DUGKS_OK) check(nullptr, rc, "create");
    try {
        check(h, dugks_gpu_init(h, c.init_kind, c.init_params.empty() ? nullptr : c.init_params.data(),
                                (int)c.init_params.size(), c.seed),
              "init");
        int64_t step = 0;
        if (!resume_file.empty()) {
            step = restore_file(h, resume_file);
            std::printf("resumed from %s at step %lld\n", resume_file.c_str(), (long long)step);
        } else {
            output(h, c, pm, out, 0);
        }
        std::printf("iteration start    cells : %d x %d    steps : %lld\n", c.grid.nx, c.grid.ny,
                    (long long)c.end_step);
        double residual = 1.0;
        while (step < c.end_step && residual > c.residual_stop) {
            // up to the next residual / output point
            int64_t n = c.residual_every - step % c.residual_every;
            const int64_t to_write = c.write_every - step % c.write_every;
            if (to_write < n) n = to_write;
            if (c.end_step - step < n) n = c.end_step - step;
            check(h, dugks_gpu_step(h, (int)n, nullptr), "step");
            step += n;
            if (step % c.residual_every == 0) {
                dugks_reductions_t r{};
                check(h, dugks_gpu_reduce(h, &r), "reduce");
                residual = r.residual;
                std::printf("%lld    %.6g    %.12e    %.6e\n", (long long)step, (double)step * c.dt, r.sum_rho,
                            r.residual);
                std::fflush(stdout);
                if (l2) append_l2(h, c, ark, out, step);
            }
            if (step % c.write_every == 0 && step < c.end_step) {
                output(h, c, pm, out, step);
                if (ac) write_profiles(h, c, out, step, false);
                if (!ckpt_file.empty()) checkpoint_file(h, ckpt_file);
            }
        }
        output(h, c, pm, out, step);
        if (ac) write_profiles(h, c, out, step, true);
        if (l2) {
            double v = 0.0;
            check(h, dugks_gpu_drop_l2(h, &v), "drop L2 norm");
            std::printf("L2_phi %.17e\n", v);
        }
        if (!ckpt_file.empty()) checkpoint_file(h, ckpt_file);
        std::printf("iteration End    step : %lld\n", (long long)step);
    } catch (...) {
        dugks_gpu_destroy(h);
        throw;
    }
    dugks_gpu_destroy(h);
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    try {
        if (argc >= 2 && std::strcmp(argv[1], "run") == 0) return run(argc, argv);
        if (argc == 4 && std::strcmp(argv[1], "rewrite-ark") == 0) {
            write_case_ark(argv[3], read_case_ark(argv[2]));
            return 0;
        }
        if (argc == 7 && std::strcmp(argv[1], "rewrite-profile") == 0) {
            const Profile k = profile_kind(argv[2]);
            const std::string text = format_profile(k, read_profile(k, std::atoi(argv[3]), std::atoi(argv[4]), argv[5]));
            std::FILE *o = std::fopen(argv[6], "wb");
            if (!o || std::fwrite(text.data(), 1, text.size(), o) != text.size() || std::fclose(o) != 0)
                throw std::runtime_error(std::string("cannot write ") + argv[6]);
            return 0;
        }
        if (argc == 4 && std::strcmp(argv[1], "rewrite-flowfield") == 0) {
            write_flowfield(argv[3], read_flowfield(argv[2]));
            return 0;
        }
        if (argc == 3 && std::strcmp(argv[1], "mesh-info") == 0) {
            const CartesianMap m = cartesian_map(read_cas(argv[2]));
            std::printf("%d %d %d\n", m.nx, m.ny, m.y_walls);
            for (size_t k = 0; k < m.cell_index.size(); ++k)
                std::printf(k + 1 < m.cell_index.size() ? "%d " : "%d\n", m.cell_index[k]);
            return 0;
        }
        if (argc == 3 && std::strcmp(argv[1], "show-config") == 0) {
            const RunConfig c = config_from_case_ark(read_case_ark(argv[2]));
            std::printf("model %d precision %d nx %d ny %d walls %d init %d nparams %zu steps %lld Mu0 %.17g "
                        "M_Phi %.17g W %.17g Sigma %.17g RhoL %.17g RhoV %.17g Gy %.17g flux %d\n",
                        c.cs.model, c.cs.precision, c.grid.nx, c.grid.ny, c.grid.y_walls, c.init_kind,
                        c.init_params.size(), (long long)c.end_step, c.cs.Mu0, c.cs.M_Phi, c.cs.W, c.cs.Sigma,
                        c.cs.RhoL, c.cs.RhoV, c.cs.Gy, c.cs.flux_scheme);
            for (double p : c.init_params) std::printf("param %.17g\n", p);
            return 0;
        }
        std::fprintf(stderr,
                     "usage: dugks_run run <Case.ark> [--out DIR] [--precision P] [--steps N] [--mesh F.cas]\n"
                     "                     [--checkpoint FILE] [--resume FILE] [--set k=v]...\n"
                     "       dugks_run rewrite-ark <in> <out>\n"
                     "       dugks_run rewrite-flowfield <in> <out>\n"
                     "       dugks_run rewrite-profile <MidX|MidY|Diag> <nx> <ny> <in> <out>\n"
                     "       dugks_run show-config <Case.ark>\n"
                     "       dugks_run mesh-info <F.cas>\n");
        return 2;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "dugks_run: %s\n", e.what());
        return 1;
    }
}
