"""Configurations of the reference build used to pin the oracle (test infrastructure).

Each variant is the unmodified reference solver compiled with one set of
compile-time switches (Ark/Constant/ZeroFlip.h), constants
(Ark/Constant/ZeroReference.h, Ark/Constant/ZeroNamespace.h,
Ark/Lib/nonidealEoS.h) and velocity model (Ark/Makefile:7), on a mesh written
by ``mesh_cas.py``.  ``consts`` holds the physical inputs; ``build_ref.py``
turns them into header substitutions and the tests turn the same numbers into
a product case, so both sides always run the same physics.

Keys of ``consts`` (all optional; absent = reference default):
  Mu0 (dynamic viscosity, Rho0 = 1 so also nu), M_Phi (mobility),
  W (interface width; Cn = W/ChLength), Sigma, RhoL, RhoV, Gy (gravity,
  enables the commented gravity line of Ark/Cpp/SourceM.cpp:32), radius,
  PP_RhoL, PP_RhoV, Tr, aCS, Tc_CS.
"""

REFERENCE_DEFAULTS = dict(Mu0=0.1, M_Phi=0.1, W=5.0, Sigma=1e-2, RhoL=10.0, RhoV=1.0,
                          Gy=0.0, radius_frac=0.36, Tr=0.85, aCS=1.0, Tc_CS=0.0943,
                          PP_RhoL=2.4806e-1, PP_RhoV=4.5435e-2, PP_radius_frac=0.25)

VARIANTS = {
    # The reference exactly as shipped: AC_Drop, D2Q9AC, 128x128 periodic.
    'ac_default': dict(model='D2Q9AC', nx=128, ny=128, walls=False, init='ac_drop',
                       consts={}),
    # Stationary droplet, 128x128 periodic, heavy phase inside (density
    # ratio 10, nu = 0.01, sigma = 1e-3, W = 4, R = 25).
    'ac_c1': dict(model='D2Q9AC', nx=128, ny=128, walls=False, init='ac_drop_inside',
                  consts=dict(Mu0=0.01, W=4.0, Sigma=1e-3, RhoL=1.0, RhoV=0.1, radius=25.0)),
    # Small non-square droplet for long, fast runs.
    'ac_small': dict(model='D2Q9AC', nx=24, ny=20, walls=False, init='ac_drop_inside',
                     consts=dict(Mu0=0.01, W=4.0, Sigma=1e-3, RhoL=1.0, RhoV=0.1, radius=6.0)),
    # HCZ pressure-based Allen-Cahn model (u != 0), periodic droplet.
    'hcz_drop': dict(model='D2Q9HCZ', nx=32, ny=32, walls=False, init='ac_drop_inside',
                     consts=dict(Mu0=0.02, W=4.0, Sigma=1e-2, RhoL=10.0, RhoV=1.0, radius=8.0)),
    # Rayleigh-Taylor: HCZ, bounce-back walls top/bottom, periodic sides,
    # gravity; Atwood 0.5 (rho 3:1).  Small box, strong gravity.
    'hcz_rt': dict(model='D2Q9HCZ', nx=16, ny=64, walls=True, init='ac_rt',
                   consts=dict(Mu0=0.01, M_Phi=0.05, W=4.0, Sigma=1e-4, RhoL=3.0, RhoV=1.0,
                               Gy=1e-4)),
    # The reference's own AC_Drop init (light bubble, case name AC_Drop) on a
    # small grid: golden Case.ark / FlowField files of the reference writers.
    'ac_ff': dict(model='D2Q9AC', nx=32, ny=24, walls=False, init='ac_drop',
                  consts=dict(Mu0=0.02, W=4.0, Sigma=1e-3, RhoL=1.0, RhoV=0.1, radius=7.0)),
    # Pseudopotential D2Q9 with the reference's own SCMP_Drop init.
    'pp_drop': dict(model='D2Q9PP', nx=32, ny=32, walls=False, init='scmp_drop', consts={}),
    # The upwind (UW) flux scheme with the 6-point cell gradients
    # (_FLUX_SCHEME_UW_ARK, Ark/Cpp/DUGKS2DSolver.cpp:540-603,689-706;
    # Ark/Lib/GradSchemeBasic.h:95-126) instead of the default CD: the small
    # periodic droplet and the HCZ droplet.  (With walls the reference's UW
    # reads the gradients of its wall shadow cells, which it never writes.)
    'uw_small': dict(model='D2Q9AC', nx=24, ny=20, walls=False, init='ac_drop_inside', scheme='UW',
                     consts=dict(Mu0=0.01, W=4.0, Sigma=1e-3, RhoL=1.0, RhoV=0.1, radius=6.0)),
    'uw_hcz': dict(model='D2Q9HCZ', nx=32, ny=32, walls=False, init='ac_drop_inside', scheme='UW',
                   consts=dict(Mu0=0.02, W=4.0, Sigma=1e-2, RhoL=10.0, RhoV=1.0, radius=8.0)),
    # UW with the reference's other cell gradients: least squares (Grad_VS_LS,
    # Ark/Lib/GradSchemeBasic.h:127-152, weights of Grad_LSMatrix :13-75) and the 4-point
    # central one (Grad_VS_4points, :76-94), the calls Ark/Cpp/DUGKS2DSolver.cpp:201-203
    # keeps commented out beside the 6-point one.
    'uwls_small': dict(model='D2Q9AC', nx=24, ny=20, walls=False, init='ac_drop_inside', scheme='UW_LS',
                       consts=dict(Mu0=0.01, W=4.0, Sigma=1e-3, RhoL=1.0, RhoV=0.1, radius=6.0)),
    'uwls_hcz': dict(model='D2Q9HCZ', nx=32, ny=32, walls=False, init='ac_drop_inside', scheme='UW_LS',
                     consts=dict(Mu0=0.02, W=4.0, Sigma=1e-2, RhoL=10.0, RhoV=1.0, radius=8.0)),
    'uw4p_hcz': dict(model='D2Q9HCZ', nx=32, ny=32, walls=False, init='ac_drop_inside', scheme='UW_4P',
                     consts=dict(Mu0=0.02, W=4.0, Sigma=1e-2, RhoL=10.0, RhoV=1.0, radius=8.0)),
    # Non-equilibrium extrapolation walls (_Wall_3_BCs_NEE, Ark/Cpp/Boundary.cpp:140-184)
    # instead of bounce-back: the Rayleigh-Taylor box and a droplet between walls.
    'nee_rt': dict(model='D2Q9HCZ', nx=16, ny=64, walls=True, init='ac_rt', wall='NEE',
                   consts=dict(Mu0=0.01, M_Phi=0.05, W=4.0, Sigma=1e-4, RhoL=3.0, RhoV=1.0, Gy=1e-4)),
    'nee_ac': dict(model='D2Q9AC', nx=24, ny=24, walls=True, init='ac_drop_inside', wall='NEE',
                   consts=dict(Mu0=0.01, W=4.0, Sigma=1e-3, RhoL=1.0, RhoV=0.1, radius=6.0)),
    # ac_ff with the UW flux scheme: golden Case.ark ("UW = Flux Scheme") and FlowField files
    'uw_ff': dict(model='D2Q9AC', nx=32, ny=24, walls=False, init='ac_drop', scheme='UW',
                  consts=dict(Mu0=0.02, W=4.0, Sigma=1e-3, RhoL=1.0, RhoV=0.1, radius=7.0)),
}
