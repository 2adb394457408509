"""Benchmark and acceptance problems as pyranda input strings.

Each problem is the mesh, EOM and IC text a pyranda user writes, plus a
``build(Sim, ...)`` helper that feeds it to any simulation class with the
pyrandaSim API (this package's, or a CPU restatement used to check it).

- Taylor-Green vortex: pyranda's examples/TaylorGreen.py (EOM and IC verbatim).
- 3-D advection of a Gaussian shell with the compact filter every stage.
- Shock-interface: Mach 1.5 planar shock into a density-ratio-3 perturbed
  interface, single-fluid Euler with LAD, one-sided closures in x, periodic
  in y and z (the structure of examples/RM3D.py without species).
- Kelvin-Helmholtz (2-D): the Euler + AFLES EOM of examples/KH.py with one
  tanh shear layer, periodic in x and walls (one-sided closures) in y; the
  ensemble benchmark advances 64 of these with seeded sizes together.
"""
import math

import numpy

# --------------------------------------------------------------- Taylor-Green
TGV_EOM = """
# Primary Equations of motion here
ddt(:rho:)  =  -ddx(:rho:*:u:)            - ddy(:rho:*:v:)               - ddz(:rho:*:w:)
ddt(:rhou:) =  -ddx(:rhou:*:u: - :tauxx:) - ddy(:rhou:*:v: - :tauxy:)    - ddz(:rhou:*:w: - :tauxz:)
ddt(:rhov:) =  -ddx(:rhov:*:u: - :tauxy:) - ddy(:rhov:*:v: - :tauyy:)    - ddz(:rhov:*:w: - :tauyz:)
ddt(:rhow:) =  -ddx(:rhow:*:u: - :tauxz:) - ddy(:rhow:*:v: - :tauyz:)    - ddz(:rhow:*:w: - :tauzz:)
ddt(:Et:)   =  -ddx( (:Et: - :tauxx:)*:u: - :tauxy:*:v: - :tauxz:*:w: )  - ddy( (:Et: - :tauyy:)*:v: -:tauxy:*:u: - :tauyz:*:w:) - ddz( (:Et: - :tauzz:)*:w: - :tauxz:*:u: - :tauyz:*:v: )
# Conservative filter of the EoM
:rho:       =  fbar( :rho:  )
:rhou:      =  fbar( :rhou: )
:rhov:      =  fbar( :rhov: )
:rhow:      =  fbar( :rhow: )
:Et:        =  fbar( :Et:   )
# Update the primatives and enforce the EOS
:u:         =  :rhou: / :rho:
:v:         =  :rhov: / :rho:
:w:         =  :rhow: / :rho:
:p:         =  ( :Et: - .5*:rho:*(:u:*:u: + :v:*:v: + :w:*:w:) ) * ( :gamma: - 1.0 )
# Artificial bulk viscosity
:ux:        =  ddx(:u:)
:vy:        =  ddy(:v:)
:wz:        =  ddz(:w:)
:div:       =  :ux: + :vy: + :wz:
# Remaining cross derivatives
:uy:        =  ddy(:u:)
:uz:        =  ddz(:u:)
:vx:        =  ddx(:v:)
:vz:        =  ddz(:v:)
:wy:        =  ddy(:w:)
:wx:        =  ddx(:w:)
:enst:      = sqrt( (:uy:-:vx:)**2 + (:uz: - :wx:)**2 + (:vz:-:wy:)**2 )
:tke:       = :rho:*(:u:*:u: + :v:*:v: + :w:*:w:)
:S:         = sqrt( :ux:*:ux: + :vy:*:vy: + :wz:*:wz: + .5*((:uy:+:vx:)**2 + (:uz: + :wx:)**2 + (:vz:+:wy:)**2) )
:mu:        =  gbar( abs(ring(:S:  )) ) * :rho: * 1.0e-4
:beta:      =  gbar( abs(ring(:div:)) * :rho: )  * 7.0e-3
:taudia:    =  (:beta:-2./3.*:mu:) *:div: - :p:
:tauxx:     =  2.0*:mu:*:ux:   + :taudia:
:tauyy:     =  2.0*:mu:*:vy:   + :taudia:
:tauzz:     =  2.0*:mu:*:wz:   + :taudia:
:tauxy:     = :mu:*(:uy:+:vx:)
:tauxz:     = :mu:*(:uz:+:wx:)
:tauyz:     = :mu:*(:vz:+:wz:)
:cs:  = sqrt( :p: / :rho: * :gamma: )
:dt: = dt.courant(:u:,:v:,:w:,:cs:)*1.0
:dt: = numpy.minimum(:dt:,0.2 * dt.diff(:beta:,:rho:))
:dt: = numpy.minimum(:dt:,0.2 * dt.diff(:mu:,:rho:))
"""

TGV_IC = """
:gamma: = 1.4
u0 = 1.0
p0 = 100.0
rho0 = 1.0
L = 1.0
:u: =  u0*sin(meshx/L)*cos(meshy/L)*cos(meshz/L)
:v: = -u0*cos(meshx/L)*sin(meshy/L)*cos(meshz/L)
:w: = 0.0*:u:
:p:  = p0 + rho0/16.0*( ( cos(2.*meshx/L) + cos(2.*meshy/L) ) * ( cos(2.*meshz/L) + 2.0 ) - 2.0 )
:rho: = rho0 + 0.0*:u:
:rhou: = :rho:*:u:
:rhov: = :rho:*:v:
:rhow: = :rho:*:w:
:Et:  = :p: / (:gamma:-1.0) + 0.5*:rho:*(:u:*:u: + :v:*:v: + :w:*:w:)
:cs:  = sqrt( :p: / :rho: * :gamma: )
:tke: = :rho:*(:u:*:u: + :v:*:v: + :w:*:w:)
:dt: = dt.courant(:u:,:v:,:w:,:cs:)
"""


# The Taylor-Green configuration of the benchmark: Mach 0.1 (p0 = rho0 u0^2 /
# (gamma M^2)), p = p0 + rho0 u0^2/16 (cos 2x + cos 2y)(cos 2z + 2), and a
# physical viscosity mu0 = rho0 u0 L / Re with Re = 1600 added to the LAD
# shear viscosity; otherwise the EOM and IC of examples/TaylorGreen.py.
TGV_RE = 1600.0
TGV_MACH = 0.1
_TGV_MU_LINE = ":mu:        =  gbar( abs(ring(:S:  )) ) * :rho: * 1.0e-4"
assert _TGV_MU_LINE in TGV_EOM
TGV_EOM_NS = TGV_EOM.replace(_TGV_MU_LINE, _TGV_MU_LINE + " + %r" % (1.0 * 1.0 * 1.0 / TGV_RE))
TGV_IC_NS = (TGV_IC.replace("p0 = 100.0\nrho0 = 1.0", "rho0 = 1.0\np0 = rho0*u0*u0/(1.4*%r*%r)" % (TGV_MACH, TGV_MACH))
             .replace("( cos(2.*meshz/L) + 2.0 ) - 2.0 )", "( cos(2.*meshz/L) + 2.0 ) )"))
assert TGV_IC_NS.count("p0 = rho0") == 1 and "2.0 ) - 2.0" not in TGV_IC_NS


def tgv_mesh(npts):
    """examples/TaylorGreen.py: periodic [0, 2 pi) in every direction."""
    return """
xdom = (0.0, 2*pi*FF,  Npts, periodic=True)
ydom = (0.0, 2*pi*FF,  Npts, periodic=True)
zdom = (0.0, 2*pi*FF,  Npts, periodic=True)
""".replace("Npts", str(npts)).replace("pi", str(math.pi)).replace("FF", str(float(npts - 1) / npts))


def build_tgv(Sim, npts, timestep, ns=False, **kw):
    """examples/TaylorGreen.py (ns=False), or the benchmark's Mach 0.1, Re 1600 configuration (ns=True)."""
    ss = Sim("TGvortex", tgv_mesh(npts), **kw)
    timestep(ss)
    ss.EOM(TGV_EOM_NS if ns else TGV_EOM)
    ss.setIC(TGV_IC_NS if ns else TGV_IC)
    return ss


# ------------------------------------------------------------ 3-D advection
ADVECTION3D_EOM = """
ddt(:phi:)  =  -ddx(:phi:) - ddy(:phi:) - ddz(:phi:)
:phi:       =  fbar( :phi: )
"""

ADVECTION3D_IC = """
r     = sqrt( (meshx-0.5)**2 + (meshy-0.5)**2 + (meshz-0.5)**2 )
:phi: = 1.0 + 0.1*exp( -(r-0.5)**2/0.1**2 )
:phi0: = 1.0*:phi:
"""


def advection3d_mesh(npts):
    """Periodic [0, 1)^3 as pyranda nodes: x1 = 0, xn = (n-1)/n."""
    xn = repr(float(npts - 1) / npts)
    return "\n".join("%sdom = (0.0, %s, %d, periodic=True)" % (ax, xn, npts) for ax in "xyz")


def build_advection3d(Sim, npts, **kw):
    ss = Sim("advection3d", advection3d_mesh(npts), **kw)
    ss.EOM(ADVECTION3D_EOM)
    ss.setIC(ADVECTION3D_IC)
    return ss


# ---------------------------------------------------------- shock-interface
# Rankine-Hugoniot state behind a Mach 1.5 shock moving in +x into gas at
# rest with rho = 1, p = 1, gamma = 1.4.
GAMMA = 1.4
MACH = 1.5
AMP = 0.05
CV = 1.0 / (GAMMA - 1.0)   # gas constant R = 1


def rankine_hugoniot(mach, gamma=GAMMA):
    """Post-shock (pressure ratio, density ratio, velocity) for a shock of Mach `mach` into rho = p = 1 at rest."""
    p_ratio = 1.0 + 2.0 * gamma / (gamma + 1.0) * (mach ** 2 - 1.0)
    rho_ratio = (gamma + 1.0) * mach ** 2 / ((gamma - 1.0) * mach ** 2 + 2.0)
    u_post = mach * math.sqrt(gamma) * (1.0 - 1.0 / rho_ratio)
    return p_ratio, rho_ratio, u_post


P_RATIO, RHO_RATIO, U_POST = rankine_hugoniot(MACH)

SHOCK_EOM = """
# Euler with LAD (the structure of examples/RM3D.py for one fluid)
ddt(:rho:)  =  -ddx(:rho:*:u:)            - ddy(:rho:*:v:)               - ddz(:rho:*:w:)
ddt(:rhou:) =  -ddx(:rhou:*:u: - :tauxx:) - ddy(:rhou:*:v: - :tauxy:)    - ddz(:rhou:*:w: - :tauxz:)
ddt(:rhov:) =  -ddx(:rhov:*:u: - :tauxy:) - ddy(:rhov:*:v: - :tauyy:)    - ddz(:rhov:*:w: - :tauyz:)
ddt(:rhow:) =  -ddx(:rhow:*:u: - :tauxz:) - ddy(:rhow:*:v: - :tauyz:)    - ddz(:rhow:*:w: - :tauzz:)
ddt(:Et:)   =  -ddx( (:Et: - :tauxx:)*:u: - :tauxy:*:v: - :tauxz:*:w: - :tx:*:kappa: )  - ddy( (:Et: - :tauyy:)*:v: -:tauxy:*:u: - :tauyz:*:w: - :ty:*:kappa: ) - ddz( (:Et: - :tauzz:)*:w: - :tauxz:*:u: - :tauyz:*:v: - :tz:*:kappa: )
:rho:       =  fbar( :rho:  )
:rhou:      =  fbar( :rhou: )
:rhov:      =  fbar( :rhov: )
:rhow:      =  fbar( :rhow: )
:Et:        =  fbar( :Et:   )
:u:         =  :rhou: / :rho:
:v:         =  :rhov: / :rho:
:w:         =  :rhow: / :rho:
:p:         =  ( :Et: - .5*:rho:*(:u:*:u: + :v:*:v: + :w:*:w:) ) * ( :gamma: - 1.0 )
:ux:        =  ddx(:u:)
:vy:        =  ddy(:v:)
:wz:        =  ddz(:w:)
:div:       =  :ux: + :vy: + :wz:
:uy:        =  ddy(:u:)
:uz:        =  ddz(:u:)
:vx:        =  ddx(:v:)
:vz:        =  ddz(:v:)
:wy:        =  ddy(:w:)
:wx:        =  ddx(:w:)
:S:         = sqrt( :ux:*:ux: + :vy:*:vy: + :wz:*:wz: + .5*((:uy:+:vx:)**2 + (:uz: + :wx:)**2 + (:vz:+:wy:)**2) )
:mu:        =  gbar( abs(ring(:S:  )) ) * :rho: * 1.0e-4
:T:         = :p: / :rho:
[:tx:,:ty:,:tz:] = grad(:T:)
LAD_CLOSURE
:taudia:    =  (:beta:-2./3.*:mu:) *:div: - :p:
:tauxx:     =  2.0*:mu:*:ux:   + :taudia:
:tauyy:     =  2.0*:mu:*:vy:   + :taudia:
:tauzz:     =  2.0*:mu:*:wz:   + :taudia:
:tauxy:     = :mu:*(:uy:+:vx:)
:tauxz:     = :mu:*(:uz:+:wx:)
:tauyz:     = :mu:*(:vz:+:wy:)
:cs:        = sqrt( :p: / :rho: * :gamma: )
:dt:        = dt.courant(:u:,:v:,:w:,:cs:)*1.0
:dt:        = numpy.minimum(:dt:,0.2 * dt.diff(:beta:,:rho:))
:dt:        = numpy.minimum(:dt:,0.2 * dt.diff(:mu:,:rho:))
# x boundaries: extrapolate the state, no transverse velocity
bc.extrap(['rho','Et','u'],['x1','xn'])
bc.const(['v','w'],['x1','xn'],0.0)
:rhou: = :rho:*:u:
:rhov: = :rho:*:v:
:rhow: = :rho:*:w:
"""

# The plain LAD closure of the bulk viscosity and conductivity (beta with the
# coefficient of the shock problem, kappa in the form of examples/KH.py:94).
PLAIN_LAD = """:beta:      =  gbar( abs(ring(:div:)) * :rho: )  * 7.0e-2
:kappa:     =  gbar( ring(:T:)* :rho:*CV/(:T: * :dt: ) ) * 1.0e-3"""
SHOCK_EOM = SHOCK_EOM.replace("LAD_CLOSURE", PLAIN_LAD.replace("CV", repr(CV)))

# Shock at x = 0.5, interface at x = 1.0 + AMP sin(2*2 pi y) sin(2*2 pi z),
# density 1 -> 3 across the interface (pressure equal), tanh profiles of
# width 2 grid spacings.
SHOCK_IC = """
:gamma: = GAMMA
delta = 2.0*DX
xs = 0.5
xi = 1.0 + AMP*sin(4.0*pi*meshy)*sin(4.0*pi*meshz)
hs = 0.5*(1.0 - tanh( (meshx - xs)/delta ))
hi = 0.5*(1.0 + tanh( (meshx - xi)/delta ))
:rho: = (1.0 + 2.0*hi)*(1.0 - hs) + RHOP*hs
:u:   = UP*hs
:v:   = 0.0*meshx
:w:   = 0.0*meshx
:p:   = 1.0 + (PP - 1.0)*hs
:rhou: = :rho:*:u:
:rhov: = :rho:*:v:
:rhow: = :rho:*:w:
:Et:  = :p:/(:gamma:-1.0) + 0.5*:rho:*(:u:*:u: + :v:*:v: + :w:*:w:)
:cs:  = sqrt( :p: / :rho: * :gamma: )
:dt:  = dt.courant(:u:,:v:,:w:,:cs:)
"""


def shock_mesh(nx, ny, nz, lx=4.0):
    """x in [0, lx] with one-sided closures; y, z periodic on [0, 1)."""
    return "\n".join([
        "xdom = (0.0, %r, %d)" % (lx, nx),
        "ydom = (0.0, %r, %d, periodic=True)" % (float(ny - 1) / ny, ny),
        "zdom = (0.0, %r, %d, periodic=True)" % (float(nz - 1) / nz, nz),
    ])


def build_shock(Sim, nx, ny, nz, packages, lx=4.0, mach=MACH, amp=AMP, eom=None, **kw):
    """The shock-interface problem; `eom` replaces SHOCK_EOM (e.g. with a learned closure)."""
    ss = Sim("shock", shock_mesh(nx, ny, nz, lx), **kw)
    packages(ss)
    ss.EOM(SHOCK_EOM if eom is None else eom)
    p_ratio, rho_ratio, u_post = rankine_hugoniot(mach)
    ic = SHOCK_IC.replace("GAMMA", repr(GAMMA)).replace("DX", repr(lx / (nx - 1))).replace("AMP", repr(amp))
    ic = ic.replace("RHOP", repr(rho_ratio)).replace("UP", repr(u_post)).replace("PP", repr(p_ratio))
    ss.setIC(ic)
    return ss


# ------------------------------------------------------------ Kelvin-Helmholtz
# examples/KH.py:8-21 constants
KH_GAMMA = 5.0 / 3.0
KH_P0 = 2.5
KH_R = 1.0
KH_CV = KH_R / (1.0 - 1.0 / KH_GAMMA) - KH_R
KH_DELTA = 1.0 / 28.0      # shear-layer thickness
KH_AMP = 0.01              # amplitude of the v perturbation
KH_SIZES = (128, 192, 256, 384, 512)

# examples/KH.py:61-99 (gamma, R0 and cv substituted by the EOM dictionary),
# with wall conditions on the y faces in the form of the shock problem's
KH_EOM = """
# Primary Equations of motion here
ddt(:rho:)  =  -ddx(:rho:*:u:)            - ddy(:rho:*:v:)
ddt(:rhou:) =  -ddx(:rhou:*:u: - :tauxx:) - ddy(:rhou:*:v: - :tauxy:)
ddt(:rhov:) =  -ddx(:rhov:*:u: - :tauxy:) - ddy(:rhov:*:v: - :tauyy:)
ddt(:Et:)   =  -ddx( (:Et: - :tauxx:)*:u: - :tauxy:*:v:  - :tx:*:kappa: )  - ddy( (:Et: - :tauyy:)*:v: -:tauxy:*:u:- :ty:*:kappa: )
# Conservative filter of the EoM
:rho:       =  fbar( :rho:  )
:rhou:      =  fbar( :rhou: )
:rhov:      =  fbar( :rhov: )
:Et:        =  fbar( :Et:   )
# Update the primatives and enforce the EOS
:u:         =  :rhou: / :rho:
:v:         =  :rhov: / :rho:
:p:         =  ( :Et: - .5*:rho:*(:u:*:u: + :v:*:v:) ) * ( gamma - 1.0 )
# Artificial bulk viscosity
:ux:        =  ddx(:u:)
:vy:        =  ddy(:v:)
:div:       =  :ux: + :vy:
# Remaining cross derivatives
:uy:        =  ddy(:u:)
:vx:        =  ddx(:v:)
:enst:      = sqrt( (:uy:-:vx:)**2 )
:tke:       = :rho:*(:u:*:u: + :v:*:v: )
:S:         = sqrt( :ux:*:ux: + :vy:*:vy:  + .5*((:uy:+:vx:)**2  ) )
:mu:        =  gbar( abs(ring(:S:  )) ) * :rho: * 1.0e-4
:beta:      =  gbar( abs(ring(:div:)) * :rho: )  * 7.0e-3
:taudia:    =  (:beta:-2./3.*:mu:) *:div: - :p:
:tauxx:     =  2.0*:mu:*:ux:   + :taudia:
:tauyy:     =  2.0*:mu:*:vy:   + :taudia:
:tauxy:     = :mu:*(:uy:+:vx:)
:T:         = :p: / (:rho: * R0 )
[:tx:,:ty:,:tz:] = grad(:T:)
:kappa:     = gbar( ring(:T:)* :rho:*cv/(:T: * :dt: ) ) * 1.0e-3
:cs:  = sqrt( :p: / :rho: * gamma )
:dt: = dt.courant(:u:,:v:,:w:,:cs:)*1.0
:dt: = numpy.minimum(:dt:,0.2 * dt.diff(:beta:,:rho:))
:dt: = numpy.minimum(:dt:,0.2 * dt.diff(:mu:,:rho:))
# y walls: extrapolate the state, no normal velocity
bc.extrap(['rho','Et','u'],['y1','yn'])
bc.const(['v'],['y1','yn'],0.0)
:rhou: = :rho:*:u:
:rhov: = :rho:*:v:
"""

# One shear layer at y = 1/2 of thickness delta: u = +-1/2, rho = 1 above and
# 2 below, uniform pressure, v' = amp sin(2 pi x) exp(-((y - 1/2)/delta)^2).
KH_IC = """
hy = tanh( (meshy-0.5)/delta )
:u: = 0.5*hy
:rho: = 1.5 - 0.5*hy
:v: = amp*sin( 2.0*pi*meshx )*exp( -((meshy-0.5)/delta)**2 )
:p: = p0 + 0.0*meshx
:Et: = :p:/( gamma - 1.0 ) + .5*:rho:*(:u:*:u: + :v:*:v:)
:rhou: = :rho:*:u:
:rhov: = :rho:*:v:
:cs:  = sqrt( :p: / :rho: * gamma )
:dt: = dt.courant(:u:,:v:,:w:,:cs:)*.1
"""


def kh_mesh(n):
    """n x n: x periodic on [0, 1) (pyranda nodes), y in [0, 1] with one-sided closures."""
    return "xdom = (0.0, %r, %d, periodic=True)\nydom = (0.0, 1.0, %d)" % (float(n - 1) / n, n, n)


def kh_sizes(count=64, seed=0):
    """Member sizes of the ensemble: n drawn uniformly from KH_SIZES by a seeded generator."""
    return [int(v) for v in numpy.random.default_rng(seed=seed).choice(list(KH_SIZES), count)]


def _kh_setup(ss, packages):
    packages(ss)
    ss.EOM(KH_EOM, {"gamma": repr(KH_GAMMA), "R0": repr(KH_R), "cv": repr(KH_CV)})
    ss.setIC(KH_IC, {"gamma": repr(KH_GAMMA), "p0": repr(KH_P0), "delta": repr(KH_DELTA),
                     "amp": repr(KH_AMP)})
    return ss


def build_kh(Sim, n, packages, **kw):
    """One n x n Kelvin-Helmholtz simulation."""
    return _kh_setup(Sim("kh", kh_mesh(n), **kw), packages)


def build_kh_ensemble(Ens, sizes, packages, **kw):
    """len(sizes) Kelvin-Helmholtz simulations, member m of size sizes[m]^2, in one ensemble."""
    return _kh_setup(Ens("kh", [kh_mesh(n) for n in sizes], **kw), packages)
