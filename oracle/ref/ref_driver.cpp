// N-step driver around the UNMODIFIED reference solver (test infrastructure).
//
// The reference's own loop stops only when the residual falls below 1e-12
// (Ark/Cpp/DUGKS2DSolver.cpp:164) and writes 12-digit text output
// (Ark/Cpp/Output.cpp:22).  This driver replaces `main` (the reference's
// main.cpp is compiled with -Dmain=reference_main so its globals stay) and
// runs a fixed number of steps, calling the reference's own phase functions
// in the order of Ark/Cpp/DUGKS2DSolver.cpp:175-327, then dumps binary FP64
// fields for the parity tests.
//
// Deliberate differences from the reference loop:
//  * fixed step count instead of the residual stop;
//  * Output_* is called only with REF_FLOWFIELD set in the environment: the
//    reference's Case.ark and FlowField writers at step 0 and after the
//    last step, and for the Allen-Cahn models its MidX / MidY / Diag profile
//    writers after the last step (Diag only when Ny >= Nx: it walks the
//    anti-diagonal (k, Nx + 1 - k), outside the grid otherwise) and, for the
//    ac_drop init, AC_Drop_L2Norm printed to stdout (golden files for the host
//    reader, writer and output tests);
//  * the pseudopotential face force (Ark/Cpp/PseudoP.cpp:39-46) reads the
//    face psi of neighbouring faces while the same loop writes them (a data
//    race at >1 thread, order-dependent at 1 thread).  Here the face loop is
//    split in two passes (all face psi first, then all face forces), the
//    defined Jacobi semantics the GPU implements;
//  * the sums and the residual are computed here in CellArray order with the
//    formulas of Ark/Cpp/DUGKS2DSolver.cpp:793-835.
//
// Usage: ref_driver <init> <steps> <dump.bin> [dump_every]
//   init: ac_drop | ac_drop_inside | ac_rt | scmp_drop | pp_noise
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "DUGKSDeclaration.h"

extern void SelfCheck();
extern int MeshConstruct(const std::string &s);
extern int MeshArea();
extern void FacesClassify();
extern void NeighbourCellConstruct();
extern void Grad_LSMatrix();
extern int MeshCheck();
extern int ShadowCellConstruct();
extern void ShadowCellCornerConstruct();
extern void DiagonalCellConstruct();
extern void CarfaceCellsConstruct();
extern void CarfaceFacesConstruct();
extern void SetFace_dxdy();
extern void AllocateResource();
extern void AC_Drop();
extern void SCMP_Drop();
extern void Update_phi_BP(Cell_2D &cell);
extern void Update_phi_fBh(Face_2D &face);
extern void Flux_2D(Face_2D &face);
extern void Update_phi_h(Face_2D &face);
extern void Update_phiFlux_h(Face_2D &face);
extern void Update_phi_T(Cell_2D &cell);
extern void Update_DVDF_Source(Cell_2D &cell);
extern void Update_DVDF_Source_h(Face_2D &face);
extern void MacroSource(Cell_2D *cellptr);
extern void Update_PseudoForce(Cell_2D &cell);
extern void Update_PseudoForce(Face_2D &face);
extern void OutputCase();
extern void Output_Flowfield(double const &t, int step);
#ifdef _ARK_ALLENCAHN_FLIP
extern void Output_MidX(int step);
extern void Output_MidY(int step);
extern void Output_Diag(int step);
extern void AC_Drop_L2Norm(double &L2_Phi);
#endif
extern void WallShadowC_fBP(Cell_2D &shadowCell);
extern void Wall_3_BB(Face_2D &face);
extern void Wall_3_NEE(Face_2D &face);
extern void Grad_VS_6points(Cell_2D *center);
extern void Grad_VS_LS(Cell_2D *center);
extern void Grad_VS_4points(Cell_2D *center);


namespace {

// 64-bit LCG (Knuth MMIX constants); the same stream is used by the product's
// host init and the CPU restatement so seeded cases agree bit for bit.
struct Lcg {
    uint64_t s;
    explicit Lcg(uint64_t seed) : s(seed) {}
    double uniform_pm1() {  // U(-1, 1) from the top 53 bits
        s = s * 6364136223846793005ULL + 1442695040888963407ULL;
        double u = static_cast<double>(s >> 11) * (1.0 / 9007199254740992.0);
        return 2.0 * u - 1.0;
    }
};

Cell_2D *cell_at(int i, int j) { return CarCellArray[i + 1][j + 1]; }

#ifdef _ARK_ALLENCAHN_FLIP
// The initialisation steps of AC_Drop (Ark/Cpp/Preprocess.cpp:705-760) with a
// caller-supplied phase-field profile.
template <class PhiFn>
void ac_init(PhiFn phi_of) {
    using PhaseFieldAC::aPhi;
    using PhaseFieldAC::bPhi;
    MacroQuantity init(Rho0, U0, V0, p0, T0, Lambda0, Mu0);
    LoopPS(Cells) {
        Cell_2D &c = CellArray[n];
        c.MsQ() = init;
        c.MsQ().Phi = phi_of(c.xc, c.yc);
        c.MsQ().Rho = aPhi * (c.MsQ().Phi) + bPhi;
        c.h.tau = PhaseFieldAC::TauMass;
        c.f.tau = c.MsQ().calcTau();
        c.Factor();
        c.FactorAC();
        Update_phi_Eq(c);
        LoopVS(DV_Qu, DV_Qv) {
            c.h.Tilde[i][j] = c.h.Eq[i][j];
            c.f.Tilde[i][j] = c.f.Eq[i][j];
        }
    }
    LoopPS(Faces) {
        Face_2D &f = FaceArray[n];
        f.MsQh() = init;
        f.h.tauh = PhaseFieldAC::TauMass;
        f.f.tauh = f.MsQh().calcTau();
        f.Factor();
        f.FactorAC();
    }
}
#endif

#ifdef _ARK_PSEUDOPSI_FLIP
// SCMP_Drop's steps (Ark/Cpp/Preprocess.cpp:337-401) with a seeded
// near-critical density field rho = rho0*(1 + amp*U(-1,1)).
void pp_noise_init(double rho0, double amp, uint64_t seed) {
    Lcg rng(seed);
    MacroQuantity init(Rho0, U0, V0, p0, T0, Lambda0, Mu0);
    std::vector<double> rho(Cells);
    for (int j = 0; j < Ny; ++j)
        for (int i = 0; i < Nx; ++i)
            rho[j * Nx + i] = rho0 * (1.0 + amp * rng.uniform_pm1());
    for (int j = 0; j < Ny; ++j)
        for (int i = 0; i < Nx; ++i) {
            Cell_2D &c = *cell_at(i, j);
            c.MsQ() = init;
            c.MsQ().Rho = rho[j * Nx + i];
            c.MsQ().p = c.MsQ().Rho * RT;
            c.MsQ().Fx = 0.0;
            c.MsQ().Fy = 0.0;
            c.f.tau = Tau0;
            c.Factor();
            Update_phi_Eq(c);
            LoopVS(DV_Qu, DV_Qv) c.f.Tilde[i][j] = c.f.Eq[i][j];
        }
    LoopPS(Faces) {
        Face_2D &f = FaceArray[n];
        f.MsQh().Fx = 0.5 * ((f.neigh->msq->Fx) + (f.owner->msq->Fx));
        f.MsQh().Fy = 0.5 * ((f.neigh->msq->Fy) + (f.owner->msq->Fy));
        f.f.tauh = Tau0;
        f.Factor();
    }
}
#endif

void run_step() {
#pragma omp parallel for schedule(static)
    for (int n = 0; n < Cells; ++n) {
        Update_phi_Eq(CellArray[n]);
#ifdef _ARK_FORCE_FLIP
        Update_DVDF_Source(CellArray[n]);
#endif
        Update_phi_BP(CellArray[n]);
    }
#ifdef _Wall_3_BCs_FLIP
#pragma omp parallel for schedule(static)
    for (int n = 0; n < WallFaceNum; ++n) WallShadowC_fBP(WallShadowCA[n]);
#endif
#ifdef _FLUX_SCHEME_UW_ARK
    // cell gradients of BarP for the UW reconstruction (Ark/Cpp/DUGKS2DSolver.cpp:196-205);
    // REF_UW_GRAD_LS / REF_UW_GRAD_4P select the gradient calls the reference keeps
    // commented out beside Grad_VS_6points (:201-203)
#pragma omp parallel for schedule(static)
    for (int n = 0; n < Cells; ++n) {
#if defined REF_UW_GRAD_LS
        Grad_VS_LS(&CellArray[n]);
#elif defined REF_UW_GRAD_4P
        Grad_VS_4points(&CellArray[n]);
#else
        Grad_VS_6points(&CellArray[n]);
#endif
    }
#endif
#if defined _ARK_PSEUDOPSI_FLIP && defined _ARK_FORCE_FLIP
    // pass 1: face distributions, moments and psi of every face
#pragma omp parallel for schedule(static)
    for (int n = 0; n < Faces; ++n) {
        Update_phi_fBh(FaceArray[n]);
        Update_MacroVar_h(FaceArray[n]);
    }
    // pass 2: face force from the psi of pass 1, then equilibrium and flux
#pragma omp parallel for schedule(static)
    for (int n = 0; n < Faces; ++n) {
        Update_PseudoForce(FaceArray[n]);
        Update_phi_Eqh(FaceArray[n]);
        Update_DVDF_Source_h(FaceArray[n]);
        Update_phi_h(FaceArray[n]);
    }
#else
#pragma omp parallel for schedule(static)
    for (int n = 0; n < InteriorFaceNum; ++n) Flux_2D(*InteriorFaceA[n]);
#ifdef _PERIODIC_12_8_BCs_FLIP
#pragma omp parallel for schedule(static)
    for (int k = 0; k < PeriodicFaceNum; ++k) Flux_2D(*PeriodicFaceA[k]);
#endif
#endif
#ifdef _Wall_3_BCs_FLIP
    // wall faces (Ark/Cpp/DUGKS2DSolver.cpp:230-250): NEE or bounce-back
#pragma omp parallel for schedule(static)
    for (int n = 0; n < WallFaceNum; ++n) {
#ifdef _Wall_3_BCs_NEE
        Wall_3_NEE(*WallFaceA[n]);
#endif
#ifdef _Wall_3_BCs_BB
        Flux_2D(*WallFaceA[n]);
        Wall_3_BB(*WallFaceA[n]);
#endif
    }
#endif
#pragma omp parallel for schedule(static)
    for (int n = 0; n < Faces; ++n) Update_phiFlux_h(FaceArray[n]);
#pragma omp parallel for schedule(static)
    for (int n = 0; n < Cells; ++n) Update_phi_T(CellArray[n]);
#pragma omp parallel for schedule(static)
    for (int n = 0; n < Cells; ++n) Update_MacroVar(CellArray[n]);
#ifdef _ARK_ALLENCAHN_FLIP
#pragma omp parallel for schedule(static)
    for (int n = 0; n < Cells; ++n) MacroSource(&CellArray[n]);
#endif
#ifdef _ARK_PSEUDOPSI_FLIP
#pragma omp parallel for schedule(static)
    for (int n = 0; n < Cells; ++n) Update_PseudoForce(CellArray[n]);
#endif
}

// Ark/Cpp/DUGKS2DSolver.cpp:807-820, CellArray order.
double residual_per_1k() {
    double SumRho2 = 0.0, SumdRho = 0.0;
    LoopPS(Cells) {
        double dRho = CellArray[n].MsQ().Rho - CellArray[n].MsQ().Rho_1k;
        SumdRho += dRho * dRho;
        SumRho2 += CellArray[n].MsQ().Rho * CellArray[n].MsQ().Rho;
        CellArray[n].MsQ().Rho_1k = CellArray[n].MsQ().Rho;
    }
    return sqrt(SumdRho / (SumRho2 + 1.0E-30));
}

double sum_rho() {  // Ark/Cpp/DUGKS2DSolver.cpp:795-803 without the [64][65] quirk
    double s = 0.0;
    LoopPS(Cells) s += CellArray[n].MsQ().Rho;
    return s;
}

void dump(const char *path, int stepno) {
    std::vector<std::string> names;
    std::vector<std::vector<double>> data;
    auto add = [&](const std::string &nm, auto getter) {
        names.push_back(nm);
        std::vector<double> v(static_cast<size_t>(Nx) * Ny);
        for (int j = 0; j < Ny; ++j)
            for (int i = 0; i < Nx; ++i) v[static_cast<size_t>(j) * Nx + i] = getter(cell_at(i, j));
        data.push_back(std::move(v));
    };
    add("rho", [](Cell_2D *c) { return c->MsQ().Rho; });
    add("u", [](Cell_2D *c) { return c->MsQ().U; });
    add("v", [](Cell_2D *c) { return c->MsQ().V; });
    add("p", [](Cell_2D *c) { return c->MsQ().p; });
    add("phi", [](Cell_2D *c) { return c->MsQ().Phi; });
    add("phix", [](Cell_2D *c) { return c->MsQ().Phi_x; });
    add("phiy", [](Cell_2D *c) { return c->MsQ().Phi_y; });
    add("rhox", [](Cell_2D *c) { return c->MsQ().Rho_x; });
    add("rhoy", [](Cell_2D *c) { return c->MsQ().Rho_y; });
    add("fx", [](Cell_2D *c) { return c->MsQ().Fx; });
    add("fy", [](Cell_2D *c) { return c->MsQ().Fy; });
    add("prevphiu", [](Cell_2D *c) { return c->MsQ().prevPhiU; });
    add("prevphiv", [](Cell_2D *c) { return c->MsQ().prevPhiV; });
    add("psi", [](Cell_2D *c) { return c->MsQ().Psi; });
    add("tauf", [](Cell_2D *c) { return c->f.tau; });
    for (int q = 0; q < DV_Qv; ++q) {
        char nm[16];
        snprintf(nm, sizeof nm, "f%d", q);
        names.push_back(nm);
        std::vector<double> v(static_cast<size_t>(Nx) * Ny);
        for (int j = 0; j < Ny; ++j)
            for (int i = 0; i < Nx; ++i) v[static_cast<size_t>(j) * Nx + i] = cell_at(i, j)->f.Tilde[0][q];
        data.push_back(std::move(v));
    }
#ifdef _ARK_ALLENCAHN_FLIP
    for (int q = 0; q < DV_Qv; ++q) {
        char nm[16];
        snprintf(nm, sizeof nm, "h%d", q);
        names.push_back(nm);
        std::vector<double> v(static_cast<size_t>(Nx) * Ny);
        for (int j = 0; j < Ny; ++j)
            for (int i = 0; i < Nx; ++i) v[static_cast<size_t>(j) * Nx + i] = cell_at(i, j)->h.Tilde[0][q];
        data.push_back(std::move(v));
    }
#endif
    FILE *fp = fopen(path, "wb");
    if (!fp) { perror(path); exit(2); }
    int32_t hdr[4] = {0x44554753, Nx, Ny, static_cast<int32_t>(names.size())};
    int64_t st = stepno;
    fwrite(hdr, sizeof hdr, 1, fp);
    fwrite(&st, sizeof st, 1, fp);
    for (auto &nm : names) {
        char buf[16] = {0};
        strncpy(buf, nm.c_str(), 15);
        fwrite(buf, 16, 1, fp);
    }
    for (auto &v : data) fwrite(v.data(), sizeof(double), v.size(), fp);
    fclose(fp);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s <init> <steps> <dump.bin> [dump_every]\n", argv[0]);
        return 2;
    }
    std::string init = argv[1];
    int nsteps = atoi(argv[2]);
    std::string dumpbase = argv[3];
    int every = argc > 4 ? atoi(argv[4]) : 0;
    std::string MeshName(_MESHFILE_NAME_ARK);
    SelfCheck();
#include "CreatMesh.h"
    AllocateResource();
    Grad_LSMatrix();
    MeshCheck();
    if (init == "ac_drop") {
        AC_Drop();
    }
#ifdef _ARK_ALLENCAHN_FLIP
    else if (init == "ac_drop_inside") {
        // heavy phase inside: phi = ½(φL+φV) + ½(φL−φV)·tanh(2(R−r)/W)
        ac_init([](double x, double y) {
            using namespace PhaseFieldAC;
            double r = sqrt((x - centerX) * (x - centerX) + (y - centerY) * (y - centerY));
            return 0.5 * (PhiL + PhiV) + 0.5 * (PhiL - PhiV) * tanh((radius - r) * 2 / wI);
        });
    } else if (init == "ac_rt") {
        // heavy (phi = PhiL) above y_i(x) = L(2 + 0.1 cos(2πx/L)), L = Lx
        ac_init([](double x, double y) {
            using namespace PhaseFieldAC;
            double yi = Lx * (2.0 + 0.1 * cos(2.0 * PI * x / Lx));
            return 0.5 * (PhiL + PhiV) + 0.5 * (PhiL - PhiV) * tanh((y - yi) * 2 / wI);
        });
    }
#endif
#ifdef _ARK_PSEUDOPSI_FLIP
    else if (init == "scmp_drop") {
        SCMP_Drop();
    } else if (init == "pp_noise") {
        const char *rc = getenv("REF_PP_RHO0");
        const char *sd = getenv("REF_PP_SEED");
        pp_noise_init(rc ? atof(rc) : 0.2, 0.01, sd ? strtoull(sd, nullptr, 10) : 12345ULL);
    }
#endif
    else {
        fprintf(stderr, "unknown init %s\n", init.c_str());
        return 2;
    }
    // REF_FLOWFIELD set: the reference's own Case.ark and FlowField writers, at
    // step 0 and after the last step (into ../FlowField relative to the cwd)
    const bool flowfield = getenv("REF_FLOWFIELD") != nullptr;
    if (flowfield) {
        OutputCase();
        Output_Flowfield(0.0, 0);
    }
    if (every > 0) dump((dumpbase + ".0").c_str(), 0);
    auto t0 = std::chrono::steady_clock::now();
    for (int s = 1; s <= nsteps; ++s) {
        run_step();
        if (s % 1000 == 0) {
            double res = residual_per_1k();
            printf("step %d sumrho %.15e residual %.15e\n", s, sum_rho(), res);
        }
        if (every > 0 && s % every == 0 && s != nsteps) dump((dumpbase + "." + std::to_string(s)).c_str(), s);
    }
    auto t1 = std::chrono::steady_clock::now();
    double secs = std::chrono::duration<double>(t1 - t0).count();
    printf("done steps %d cells %d seconds %.6f mlups %.4f sumrho %.15e\n", nsteps, Cells, secs,
           nsteps > 0 ? 1e-6 * Cells * (double)nsteps / secs : 0.0, sum_rho());
    dump(dumpbase.c_str(), nsteps);
    if (flowfield) {
        Output_Flowfield(nsteps * dt, nsteps);
#ifdef _ARK_ALLENCAHN_FLIP
        Output_MidX(nsteps);
        Output_MidY(nsteps);
        if (Ny >= Nx) Output_Diag(nsteps);
        if (init == "ac_drop") {
            double l2 = 0.0;
            AC_Drop_L2Norm(l2);
            printf("L2_phi %.17e\n", l2);
        }
#endif
    }
    return 0;
}
