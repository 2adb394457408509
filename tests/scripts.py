"""The reference's regression scripts, restated as functions of a simulation class.

Each function follows one script of pyranda/examples (the ones its test-suite
runs, tests/cases/*.py) and returns the scalar the script prints last.  The
simulation class is either the oracle's numpy restatement (``OracleSim``) or
the product's ``pyranda_gb300.pyrandaSim``; the scripts only use the API the
two share.  Mesh and EOM strings are the reference scripts' own inputs.
"""
import numpy

from pyranda_gb300.problems import TGV_EOM, TGV_IC, tgv_mesh  # noqa: F401  (problem strings)


def _f(x):
    """float() of a Python number, numpy scalar or 0-d torch tensor."""
    try:
        return float(x)
    except TypeError:
        return float(x.item())


def _sumsq_diff(a, b):
    d = a - b
    s = (d * d).sum()
    return _f(s)


def unit_test(Sim, **kw):
    """examples/unit_test.py: derivatives and filters on periodic and one-sided meshes."""
    ERROR = 0.0
    Nx = 32
    L = numpy.pi * 2.0 * (Nx - 1) / Nx
    domain = """
xdom = (0.0 , L , Nx ,periodic=True)
ydom = (0.0 , L , Nx ,periodic=True)
zdom = (0.0 , L , Nx ,periodic=True)
""".replace("L", str(L)).replace("Nx", str(Nx))
    pysim = Sim("advection", domain, **kw)
    expr = "sum( abs( ddx( sin(meshx) ) - cos(meshx) ))"
    for e in (expr, expr.replace("x", "y"), expr.replace("x", "z")):
        ERROR += _f(pysim.eval(e))
    domain = """
xdom = (0.0 , 1.0 , Nx )
ydom = (0.0 , 1.0 , Nx )
zdom = (0.0 , 1.0 , Nx )
""".replace("Nx", str(Nx))
    pysim2 = Sim("nonperiodic", domain, **kw)
    for expr in ("mean( abs(ddx(meshx*0.0)) )", "mean( abs(ddx(meshx*0.0 + 1.0)) )"):
        for e in (expr, expr.replace("x", "y"), expr.replace("x", "z")):
            ERROR += _f(pysim2.eval(e))
    expr = "mean( abs(ddx(meshx**power) - power*meshx**(power-1) )  )"
    for power in (1, 2, 3, 4):
        ex = expr.replace("power", str(float(power)))
        for e in (ex, ex.replace("x", "y"), ex.replace("x", "z")):
            ERROR += _f(pysim2.eval(e))
    groups = [
        (pysim2, ["mean( abs(fbar(meshx*0.0)) )", "mean( abs(fbar(meshx*0.0 + 1.0) - (meshx*0.0 + 1.0)  ) )",
                  "mean( abs(fbar(meshx) - (meshx)  ) )"]),
        (pysim, ["mean( abs(fbar(sin(meshx)) - sin(meshx)  ) )", "mean( abs(fbar( meshx*0.0 + 1.0) - 1.0  ) )",
                 "mean( abs(fbar( meshx*0.0 )  ) )"]),
        (pysim2, ["mean( abs(gbar(meshx*0.0)) )", "mean( abs(gbar(meshx*0.0 + 1.0) - (meshx*0.0 + 1.0)  ) )",
                  "mean( abs(gbar(meshx) - (meshx)  ) )"]),
        (pysim, ["mean( abs(gbar(sin(meshx)) - sin(meshx)  ) )", "mean( abs(gbar( meshx*0.0 + 1.0) - 1.0  ) )",
                 "mean( abs(gbar( meshx*0.0 )  ) )"]),
    ]
    for sim, exprs in groups:
        for e in exprs:
            ERROR += _f(sim.eval(e))
    return ERROR


def advection_1d(Sim, Npts, **kw):
    """examples/advection.py N 1: one period of periodic advection, sum of squared error."""
    L = numpy.pi * 2.0
    Lp = L * (Npts - 1.0) / Npts
    ss = Sim("advection", "xdom = (0.0, %s, %d, periodic=True)" % (repr(Lp), Npts), **kw)
    ss.EOM(" ddt(:phi:)  =  -:c: * ddx(:phi:) ")
    ss.setIC("""
r   = sqrt( (meshx-pi)**2  )
:phi: = 1.0 + 0.1 * exp( -(r/(pi/4.0))**2 )
:phi2: = 1.0*:phi:
:c:   = 1.0
""")
    v = 1.0
    dt_max = v / Npts * L * .90
    tt = L / v * 1.0
    dt = dt_max
    time = 0.0
    while tt > time:
        time = ss.rk4(time, dt)
        dt = min(dt_max, (tt - time))
    return _sumsq_diff(ss.variables["phi"].data, ss.variables["phi2"].data)


def make_tgv(Sim, Npts, timestep, **kw):
    from pyranda_gb300.problems import build_tgv
    return build_tgv(Sim, Npts, timestep, **kw)


def taylor_green(Sim, Npts, tstop, timestep, steps=None, **kw):
    """examples/TaylorGreen.py N 1: enstrophy ratio at t = tstop (CFL 0.5)."""
    ss = make_tgv(Sim, Npts, timestep, **kw)
    CFL = 0.5
    dt = ss.variables["dt"].data * CFL
    enst0 = ss.var("enst").sum()
    time = 0.0
    n = 0
    while (time < tstop) if steps is None else (n < steps):
        time = ss.rk4(time, dt)
        dt = ss.variables["dt"].data * CFL
        n += 1
    return _f(ss.var("enst").sum() / enst0)


EULER_1D = """
# Primary Equations of motion here
ddt(:rho:)  =  -ddx(:rho:*:u:)
ddt(:rhou:) =  -ddx(:rhou:*:u: + :p: - :tau:)
ddt(:Et:)   =  -ddx( (:Et: + :p: - :tau:)*:u: )
# Conservative filter of the EoM
:rho:       =  fbar( :rho:  )
:rhou:      =  fbar( :rhou: )
:Et:        =  fbar( :Et:   )
# Update the primatives and enforce the EOS
:u:         =  :rhou: / :rho:
:p:         =  ( :Et: - .5*:rho:*(:u:*:u:) ) * ( :gamma: - 1.0 )
# Artificial bulk viscosity (old school way)
:div:       =  ddx(:u:)
:beta:      =  gbar(abs(ring(:div:))) * :rho: * 7.0e-2
:tau:       =  :beta:*:div:
"""


def shu_osher_run(Sim, Npts, packages, graphs=False, **kw):
    """getShu of examples/shu_osher.py: returns (x, rho) at t = 1.8 (graphs: each
    RK step replayed from a CUDA graph, bit-identical to eager)."""
    L = 10.0
    Lp = L * (Npts - 1.0) / Npts
    imesh = "xdom = (-Lp/2.0, Lp/2.0, Npts)".replace("Lp", str(Lp)).replace("Npts", str(Npts))
    ss = Sim("sod", imesh, **kw)
    packages(ss)
    eom = EULER_1D + """
# Apply constant BCs
bc.const(['u'],['xn'],0.0)
bc.const(['u'],['x1'],2.629369)
bc.const(['rho'],['x1'],3.857143)
bc.const(['p'],['x1'],10.33333)
bc.const(['Et'],['x1'],39.166585)
:rhou: = :rho:*:u:
:cs:  = sqrt( :p: / :rho: * :gamma: )
:dt: = dt.courant(:u:,0.0,0.0,:cs:)
:dt: = numpy.minimum(:dt:,0.2 * dt.diff(:beta:,:rho:))
"""
    ss.EOM(eom)
    ic = """
:gamma: = 1.4
eps = 2.0e-1
:tmp: = (meshx+4.0)/%s
:dum: = tanh(:tmp:)
:dum: = (:dum:+1.0)/2.0
:rho: = 3.857143 + :dum:*(1.0+eps*sin(5.0*meshx) - 3.857143)
:u: = 2.629369*(1.0-:dum:)
:p: = 10.33333 + :dum:*(1.0-10.33333)
:rhou: = :rho: * :u:
:Et:  = :p:/(:gamma: -1.0) + .5*:rho:*:u:*:u:
"""
    ss.setIC(ic % ss.dx)
    if graphs:
        ss.use_graphs(True)
    time = 0.0
    CFL = 0.5
    dt = _f(ss.variables["dt"].data) * CFL * .01
    tt = 1.8
    while tt > time:
        time = ss.rk4(time, dt)
        dt = min(dt * 1.1, _f(ss.variables["dt"].data) * CFL)
        dt = min(dt, (tt - time))
    x = _host(ss.variables["meshx"].data if "meshx" in ss.variables else ss.meshx)[:, 0, 0]
    rho = _host(ss.variables["rho"].data)[:, 0, 0]
    return x, rho


def _meshx(ss):
    """x coordinates of the mesh (ss.mesh.coords[0] in pyranda; the oracle keeps them as ss.meshx)."""
    return ss.variables["meshx"].data if "meshx" in ss.variables else ss.meshx


def _host(a):
    if hasattr(a, "cpu"):
        t = a.detach()
        return numpy.asfortranarray(t.permute(2, 1, 0).cpu().numpy().transpose(2, 1, 0))
    if hasattr(a, "data") and not isinstance(a, numpy.ndarray):
        return _host(a.data)
    return numpy.asarray(a)


def shu_osher(Sim, packages, graphs=False, **kw):
    """examples/shu_osher.py 1: average convergence rate of rho(1.85) over N = 100..800."""
    sol = []
    for n in (100, 200, 400, 800):
        x, rho = shu_osher_run(Sim, n, packages, graphs=graphs, **kw)
        sol.append(numpy.interp(1.85, x, rho))
    sol = numpy.array(sol)
    diff = numpy.abs(sol[1:] - sol[:-1])
    cr1 = numpy.log(diff[-1] / diff[-2]) / numpy.log(.5)
    cr2 = numpy.log(diff[-2] / diff[-3]) / numpy.log(.5)
    return float((cr1 + cr2) / 2.0)


EULER_2D = """
# Primary Equations of motion here
ddt(:rho:)  =  -ddx(:rho:*:u:)                  - ddy(:rho:*:v:)
ddt(:rhou:) =  -ddx(:rhou:*:u: + :p: - :tau:)   - ddy(:rhou:*:v:)
ddt(:rhov:) =  -ddx(:rhov:*:u:)                 - ddy(:rhov:*:v: + :p: - :tau:)
ddt(:Et:)   =  -ddx( (:Et: + :p: - :tau:)*:u: ) - ddy( (:Et: + :p: - :tau:)*:v: )
# Conservative filter of the EoM
:rho:       =  fbar( :rho:  )
:rhou:      =  fbar( :rhou: )
:rhov:      =  fbar( :rhov: )
:Et:        =  fbar( :Et:   )
# Update the primatives and enforce the EOS
:u:         =  :rhou: / :rho:
:v:         =  :rhov: / :rho:
:p:         =  ( :Et: - .5*:rho:*(:u:*:u: + :v:*:v:) ) * ( :gamma: - 1.0 )
# Artificial bulk viscosity (old school way)
:div:       =  ddx(:u:) + ddy(:v:)
:beta:      =  gbar(abs(ring(:div:))) * :rho: * 7.0e-2
:tau:       =  :beta:*:div:
# Apply constant BCs
bc.extrap(['rho','Et'],['x1','xn','y1','yn'])
bc.const(['u','v'],['x1','xn','y1','yn'],0.0)
"""


def euler_2d(Sim, Npts, packages, **kw):
    """examples/euler.py N 1 (tests/cases/test2deuler.py): the 2-D Sod problem
    (a circular shock tube) on an N x N one-sided mesh to t = 2 pi / 8; returns
    (x, rho) along the middle row j = N/2, the profile the test compares."""
    L = numpy.pi * 2.0
    Lp = L * (Npts - 1.0) / Npts
    mesh = ("xdom = (0.0, %r, %d)\nydom = (0.0, %r, %d)\nzdom = (0.0, %r, 1, periodic=True)"
            % (Lp, Npts, Lp, Npts, Lp))
    ss = Sim("advection", mesh, **kw)
    packages(ss)
    ss.EOM(EULER_2D)
    ss.setIC("""rad = sqrt( (meshx-pi)**2  +  (meshy-pi)**2 )
:gamma: = 1.4
:Et:  = gbar( where( rad < pi/2.0, 1.0/(:gamma:-1.0) , .1 /(:gamma:-1.0) ) )
:rho: = gbar( where( rad < pi/2.0, 1.0    , .125 ) )
""")
    time = 0.0
    v = 1.0
    dt_max = v / Npts * 0.75
    tt = L / v * .125
    dt = dt_max
    while tt > time:
        time = ss.rk4(time, dt)
        dt = min(dt_max, (tt - time))
    x = _host(_meshx(ss))[:, Npts // 2, 0]
    rho = _host(ss.variables["rho"].data)[:, Npts // 2, 0]
    return x, rho


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
"""

KH_IC = """
Um = (u1-u2)/2.0
rhoM = (rho1-rho2)/2.0
:u: =                     u1-Um*exp( -(meshy-.75)/L)
:u: = where( meshy < .75, u2+Um*exp( -(.75-meshy)/L) , :u: )
:u: = where( meshy < .50, u2+Um*exp( (-meshy+.25)/L) , :u: )
:u: = where( meshy < .25, u1-Um*exp(  (meshy-.25)/L) , :u: )
:v: = 0.01*sin( 4.*pi*meshx ) + Vmean
:rho: =                     rho1-rhoM*exp( -(meshy-.75)/L)
:rho: = where( meshy < .75, rho2+rhoM*exp( -(.75-meshy)/L) , :rho: )
:rho: = where( meshy < .50, rho2+rhoM*exp( (-meshy+.25)/L) , :rho: )
:rho: = where( meshy < .25, rho1-rhoM*exp(  (meshy-.25)/L) , :rho: )
:p: += p0
# Form conserved variables
:Et: = :p:/( gamma - 1.0 ) + .5*:rho:*(:u:*:u: + :v:*:v:)
:rhou: = :rho:*:u:
:rhov: = :rho:*:v:
:cs:  = sqrt( :p: / :rho: * gamma )
:dt: = dt.courant(:u:,:v:,:w:,:cs:)*.1
"""


def kelvin_helmholtz_2d(Sim, Npts, packages, tfinal=1.5, **kw):
    """examples/KH.py N 0 <name> 1 (tests/cases/test2deuler.py:47-51): the
    McNally et al. Kelvin-Helmholtz problem with the AFLES terms on a periodic
    N x N mesh to t = 1.5; returns (x, rho) along row j = 3N/4, the profile the
    test compares."""
    gamma, p0, u1, u2, rho1, rho2, L, tFinal, R = 5. / 3., 2.5, 0.5, -0.5, 1.0, 2.0, 0.025, tfinal, 1.0
    Vmean = 0.0
    cp = R / (1.0 - 1.0 / gamma)
    cv = cp - R
    dt_max = 1.0
    mesh = """
xdom = (0.0, len,  Npts, periodic=True)
ydom = (0.0, len,  Npts, periodic=True)
""".replace("Npts", str(Npts)).replace("len", str(1.0 * (Npts - 1.0) / Npts))
    ss = Sim("KelvinHelmholtz", mesh, **kw)
    packages(ss)
    ss.EOM(KH_EOM, {"gamma": gamma, "R0": R, "cv": cv})
    ss.setIC(KH_IC, {"gamma": gamma, "u1": u1, "u2": u2, "p0": p0, "rho1": rho1, "rho2": rho2, "L": L,
                     "Vmean": Vmean})
    time = 0.0
    dt = _f(ss.variables["dt"].data)
    while tFinal > time:
        time = ss.rk4(time, dt)
        dt = min(_f(ss.variables["dt"].data), 1.1 * dt)
        dt = min(dt_max, dt)
        dt = min(dt, (tFinal - time))
    j = int(3 * Npts / 4)
    x = _host(_meshx(ss))[:, j, 0]
    rho = _host(ss.variables["rho"].data)[:, j, 0]
    return x, rho


def profile_error(golden_path, x, v):
    """tests/testObj.py:checkProfile: max |base - test| / max |base| over the
    common length of the two profiles (row 1 of the baseline file)."""
    base = numpy.loadtxt(golden_path)
    m = min(base.shape[1], len(v))
    return float(numpy.max(numpy.abs(base[1, :m] - numpy.asarray(v)[:m])) / numpy.max(numpy.abs(base[1, :m])))


EULER_RZ_EOM = """
# Primary Equations of motion here
ddt(:rho:)  =  -:mass:
ddt(:rhou:) =  -:xmom:
ddt(:rhow:) =  -:zmom:
ddt(:Et:)   =  -div( (:Et: + :p: - :tau:)*:u:,:v:, (:Et: + :p: - :tau:)*:w: )
# Conservative filter of the EoM
:rho:       =  fbar( :rho:  )
:rhou:      =  fbar( :rhou: )
:rhow:      =  fbar( :rhow: )
:Et:        =  fbar( :Et:   )
# Update the primatives and enforce the EOS
:u:         =  :rhou: / :rho:
:w:         =  :rhow: / :rho:
:p:         =  ( :Et: - .5*:rho:*(:u:*:u: + :w:*:w:) ) * ( :gamma: - 1.0 )
# Artificial bulk viscosity (old school way)
:div:       =  div(:u:,:v:,:w:)
:beta:      =  gbar(abs(ring(:div:))) * :rho: * 7.0e-2
:tau:       =  :beta:*:div:
:v:         = :v: * 0.0
# Compute divT of momentum
:mass: = div(:rho:*:u:               , :v:, :rho:*:w:)
[:fxx:,:fxy:,:fxz:] = [:rhou:*:u: + :p: - :tau:, :v:, :rhou:*:w:]
[:fyx:,:fyy:,:fyz:] = [      :v:               , :p:-:tau: , :v:       ]
[:fzx:,:fzy:,:fzz:] = [:rhow:*:u:,               :v:, :rhow:*:w: + :p: - :tau:]
[:xmom:,:ymom:,:zmom:] = divT(:fxx:,:fxy:,:fxz:,:fyx:,:fyy:,:fyz:,:fzx:,:fzy:,:fzz:)
"""


def euler_rz(Sim, Npts, packages, **kw):
    """examples/eulerRZ.py N 1 (tests/cases/test2deuler.py euler-RZ-128): a
    cylindrical (r, z) Sod problem with a symmetry plane at the axis, run to
    t = 0.5; returns (r, p) with p along z at r index N/2, the profile the
    test compares."""
    L = numpy.pi * 2.0
    dx2 = L / (Npts - 1) / 2.0
    opts = {"coordsys": 1, "periodic": [False, False, True], "x1": [dx2, -0.1, 0.0], "xn": [L, 0.1, L],
            "nn": [Npts, 1, Npts], "symmetric": [[True, False], [False, False], [False, False]]}
    ss = Sim("advection", opts, **kw)
    packages(ss)
    ss.EOM(EULER_RZ_EOM)
    ss.setIC("""rad = sqrt( (meshx-pi)**2  +  (meshz-pi)**2 )
:gamma: = 1.4
wgt = .5*(1.0-tanh( (rad-pi/2.0)/.1) )   # [0,1]
:Et:  = 1.0/(:gamma:-1.0) * (wgt*.9 + .1)
:rho: = 1.0*wgt + (1.0-wgt)*.125
""")
    time = 0.0
    dt_max = 1.0 / Npts * 0.75
    tt = 0.5
    dt = dt_max
    while tt > time:
        time = ss.rk4(time, dt)
        dt = min(dt_max, (tt - time))
    half = int(Npts / 2.0)
    x = _host(_meshx(ss))[:, 0, 0]
    p = _host(ss.variables["p"].data)[half, 0, :]
    return x, p


SPH_DT = """
:cs:  = sqrt( :p: / :rho: * :gamma: )
:dt: = dt.courant(:u:,:v:,:w:,:cs:)
"""

SPH_IC = """rad = sqrt( (meshx-pi)**2  +  (meshy-0.0)**2 )
:gamma: = 1.4
wgt = .5*(1.0-tanh( (rad-pi/16.0)/.1) )   # [0,1]
:Et:  = 1.0/(:gamma:-1.0) * (wgt*.9 + .1)
:rho: = 1.0*wgt + (1.0-wgt)*.125
"""


def _native(ss, q):
    """ss.mesh.coordsNative[q] (pyrandaMesh.py:176-191), on the host."""
    return _host(ss.mesh.coordsNative[q] if hasattr(ss, "mesh") else ss.coordsNative[q])


def _sph_run(ss, dt_max, tt):
    time = 0.0
    dt = dt_max
    while tt > time:
        time = ss.rk4(time, dt)
        dt = min(dt_max, _f(ss.variables["dt"].data))
        dt = min(dt, (tt - time))


def euler_sph_1d(Sim, Npts, packages, **kw):
    """examples/eulerSpherical1D.py N 1 (tests/cases/test2deuler.py euler-SPH-1D):
    a spherical Sod problem on 4N radial points (coordsys 2, one point in theta
    and phi) to t = 0.1, with the courant and diffusion limits; returns
    (r, p), the profile the test compares."""
    L = numpy.pi * 2.0
    spike = numpy.pi / 16
    Mpts = Npts * 4
    x0 = L / Mpts
    opts = {"coordsys": 2, "periodic": [False, False, True], "x1": [x0, numpy.pi / 2 - .01, 0 * numpy.pi - spike],
            "xn": [L, numpy.pi / 2 + .01, 0 * numpy.pi + spike], "nn": [Mpts, 1, 1]}
    ss = Sim("sod2dSpherical_1D", opts, **kw)
    packages(ss)
    eom = EULER_RZ_EOM + SPH_DT + ":dt: = numpy.minimum( :dt:, 0.1 * dt.diff(:beta:,:rho:) )\n"
    eom += ":rhow: = :rhow: * 0.0\n"
    eom += "bc.const(['u'],['x1'],0.0) \n"
    eom += "bc.extrap(['rho','p'],['x1'],order=1) \n"
    eom += ":rhou: = :rho:*:u: \n"
    eom += ":Et: = :p:/( :gamma: - 1.0 ) + .5*:rho:*(:u:*:u: + :w:*:w:) \n"
    ss.EOM(eom)
    ss.setIC(SPH_IC)
    _sph_run(ss, 1.0 / ss.nx * 0.05, 0.1)
    p = _host(ss.variables["p"].data)[:, 0, 0]
    return _native(ss, 0)[:, 0, 0], p


def euler_sph_2d(Sim, Npts, packages, **kw):
    """examples/eulerSpherical.py N 1 (tests/cases/test2deuler.py euler-SPH-2D):
    the spherical Sod problem on 4N radii x N angles phi (coordsys 2) to t =
    0.1; returns (r, rho averaged over phi), the profile the test compares."""
    L = numpy.pi * 2.0
    spike = numpy.pi / 16
    opts = {"coordsys": 2, "periodic": [False, False, True], "x1": [L / 10, numpy.pi / 2 - .01, 0 * numpy.pi - spike],
            "xn": [L, numpy.pi / 2 + .01, 0 * numpy.pi + spike], "nn": [Npts * 4, 1, Npts]}
    ss = Sim("sod2dSpherical", opts, **kw)
    packages(ss)
    ss.EOM(EULER_RZ_EOM + "bc.const(['u'],['x1','xn'],0.0)\n" + SPH_DT)
    ss.setIC(SPH_IC)
    _sph_run(ss, 1.0 / ss.nx * 0.05, 0.1)
    rho = _host(ss.variables["rho"].data)[:, 0, :].mean(axis=1)
    return _native(ss, 0)[:, 0, int(Npts / 2)], rho


OMESH_EOM = """
ddt(:rho:)  =  -div(:rho:*:u:,  :rho:*:v:)
ddt(:rhou:) =  -div(:rhou:*:u: + :p: - :tau:, :rhou:*:v:)
ddt(:rhov:) =  -div(:rhov:*:u:, :rhov:*:v: + :p: - :tau:)
ddt(:Et:)   =  -div( (:Et: + :p: - :tau:)*:u: , (:Et: + :p: - :tau:)*:v:  )
:rho:       =  fbar( :rho:  )
:rhou:      =  fbar( :rhou: )
:rhov:      =  fbar( :rhov: )
:Et:        =  fbar( :Et:   )
:u:         =  :rhou: / :rho:
:v:         =  :rhov: / :rho:
:p:         =  ( :Et: - .5*:rho:*(:u:*:u: + :v:*:v:) ) * ( :gamma: - 1.0 )
:div:       =  div(:u:,:v:)
:beta:      =  gbar( ring(:div:) * :rho: ) * 7.0e-2
:tau:       = :beta:*:div:
bc.extrap(['u','v','rho','p'],['yn'])
bc.const(['u'],['yn'],u0)
bc.const(['v'],['yn'],0.0)
bc.extrap(['rho','p'],['y1'])
bc.slip([ ['u','v']  ],['y1'])
:Et:  = :p: / ( :gamma: - 1.0 )  + .5*:rho:*(:u:*:u: + :v:*:v:)
:rhou: = :rho:*:u:
:rhov: = :rho:*:v:
:cs:  = sqrt( :p: / :rho: * :gamma: )
:dt: = dt.courant(:u:,:v:,:w:,:cs:)
:dtB: = dt.diff(:beta:,:rho:)
:umag: = sqrt( :u:*:u: + :v:*:v: )
"""

OMESH_IC = """
:gamma: = 1.4
:R: = 1.0
:cp: = :R: / (1.0 - 1.0/:gamma: )
:cv: = :cp: - :R:
rad = sqrt( meshx**2  +  meshy**2 )
:rho: = 1.0 + 3d()
:p:  =  1.0 + 3d()
:u: = mach * sqrt( :p: / :rho: * :gamma:)
:v: = 0.0 + 3d()
:Et: = :p:/( :gamma: - 1.0 ) + .5*:rho:*(:u:*:u: + :v:*:v:)
:rhou: = :rho:*:u:
:rhov: = :rho:*:v:
:cs:  = sqrt( :p: / :rho: * :gamma:)
:dt: = dt.courant(:u:,:v:,:w:,:cs:)
"""


def cylinder_omesh(Sim, Npts, packages, tt=3.0, **kw):
    """examples/cylinder_curv2.py N 1 (tests/cases/testCylinder.py
    cylinder_omesh-2d-64): Mach 1.5 flow past a cylinder on a curvilinear
    O-mesh (coordsys 3; periodic around, slip wall at the cylinder, inflow
    and extrapolation at the far edge) to t = 3; returns (x, |u|) along the
    middle radial line j = N/2, the profile the test compares."""
    L = numpy.pi * 2.0
    Lp = L * (Npts - 1.0) / Npts
    Ri, Rf = 1.0, 10.0
    NX = NY = Npts

    def cyl_mesh(i, j, k):
        theta = float(i) / float(NX) * 2.0 * numpy.pi
        r = float(j) / float(NY - 1) * (Rf - Ri) + Ri
        return r * numpy.cos(theta), r * numpy.sin(theta), 0.0

    opts = {"coordsys": 3, "function": cyl_mesh, "periodic": [True, False, False], "periodicGrid": False,
            "x1": [-2 * Lp, -2 * Lp, 0.0], "xn": [2 * Lp, 2 * Lp, Lp], "nn": [NX, NY, 1]}
    ss = Sim("cylinder_omesh", opts, **kw)
    packages(ss)
    rho0, p0, gamma, mach = 1.0, 1.0, 1.4, 1.5
    u0 = numpy.sqrt(p0 / rho0 * gamma) * mach
    ss.EOM(OMESH_EOM.replace("u0", str(u0)).replace("p0", str(p0)).replace("rho0", str(rho0)))
    ss.setIC(OMESH_IC.replace("mach", str(mach)))
    time = 0.0
    CFL = 0.8
    dt = _f(ss.variables["dt"].data) * CFL * .1
    while tt > time:
        time = ss.rk4(time, dt)
        dt = _f(ss.variables["dt"].data) * CFL
        dt = min(dt, 1.1 * dt)
        dt = min(0.2 * _f(ss.variables["dtB"].data), dt)
        dt = min(dt, (tt - time))
    x = _host(_meshx(ss))[:, :, 0]
    v = _host(ss.variables["umag"].data)[:, :, 0]
    return x[:, int(NY / 2)], v[:, int(NY / 2)]


def heat_1d(Sim, Npts, packages, **kw):
    """examples/heat1D.py N 1 (tests/cases/testHeat1D.py heat1D-analytic-N):
    the heat equation ddt(phi) = c lap(phi) on a one-sided line with constant
    end values, started from its linear steady state and run 500 steps;
    returns sum |phi - analytic| (the golden is 0 within 1e-4)."""
    L = numpy.pi * 2.0
    Lp = L * (Npts - 1.0) / Npts
    opts = {"coordsys": 0, "periodic": [False, True, True], "x1": [0.0, 0.0, 0.0], "xn": [Lp, Lp, Lp],
            "nn": [Npts, 1, 1]}
    ss = Sim("heat_equation", opts, **kw)
    packages(ss)
    ss.EOM("""
ddt(:phi:)  =  :c: * lap(:phi:)
bc.const(['phi'],['x1'],2.0)
bc.const(['phi'],['xn'],1.0)
""")
    ss.setIC("""
xnn = meshx[-1,0,0]
:phi: = 1.0 + 1.0*(xnn - meshx)/xnn
:c:   = 1.0
""")
    x = _host(_meshx(ss))[:, 0, 0]
    dt_max = L / Npts * .005
    tt = dt_max * 500
    dt = dt_max
    time = 0.0
    while tt > time:
        time = ss.rk4(time, dt)
        dt = min(dt_max, (tt - time))
    xnn = x[-1]
    anl = 1.0 + 1.0 * (xnn - x) / xnn
    return float(numpy.sum(numpy.abs(anl - _host(ss.variables["phi"].data)[:, 0, 0])))


def integration(Sim, Npts, **kw):
    """examples/intTest.py N 1 (tests/cases/testIntegration.py integration-N):
    ddt(a) = a and ddt(b) = cos(6 simtime) on one point with dt = 1/N to
    t = 1; returns sum |a - (1 - a0 + e^t)| over the steps, which measures
    the LSRK(5,4) scheme and its stage times."""
    ss = Sim("integralTests", "xdom = (0.0 , 1.0 , 1 )", **kw)
    ss.EOM("""
ddt(:a:)  =  :a:
ddt(:b:)  =  cos( 6.0*simtime )
""")
    a0, b0 = 1.0, 0.0
    ss.setIC("""
:a: = %s
:b: = %s
""" % (a0, b0))
    dt = 1.0 / float(Npts)
    time = 0.0
    tt, aa = [time], [a0]
    while time < 1.0:
        time = ss.rk4(time, dt)
        tt.append(time)
        aa.append(float(_host(ss.variables["a"].data)[0, 0, 0]))
    tt, aa = numpy.array(tt), numpy.array(aa)
    return float(numpy.sum(numpy.abs(aa - (1.0 - a0 + numpy.exp(tt)))))
