"""Small parity configurations shared by the fixture generator and the tests.

Faces are plbpd's: east/west bound x, north/south bound y, up/down bound z.
D2Q9 lives in the x-z plane (ny = 1).
"""

CASES = {
    # D2Q9 channel: periodic in x, walls up/down, moving lid, body force
    "d2q9_channel": dict(model="D2Q9", nx=8, ny=1, nz=6, nu=0.1, rho0=1.0, u0=(0.0, 0.0, 0.0),
                         force=(1e-5, 0.0, 0.0), rho_solid=1.0,
                         face_type={"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"},
                         face_vel={"up": (0.05, 0.0, 0.0), "down": (0.0, 0.0, 0.0)}),
    # D3Q19, x and y periodic, z walls (the Couette3D layout, src/Flow.cpp:41-62)
    "d3q19_xy_periodic": dict(model="D3Q19", nx=8, ny=7, nz=6, nu=0.5, rho0=1.0, u0=(0.01, 0.0, 0.0),
                              force=(0.0, 0.0, 0.0), rho_solid=1.0,
                              face_type={"east": "periodic", "west": "periodic", "north": "periodic",
                                         "south": "periodic", "up": "noslip", "down": "noslip"},
                              face_vel={"up": (0.05, 0.0, 0.0), "down": (0.0, 0.0, 0.0)}),
    # D3Q27 square duct: periodic x, walls on y and z, two moving walls
    "d3q27_duct": dict(model="D3Q27", nx=6, ny=5, nz=7, nu=0.05, rho0=1.0, u0=(0.0, 0.01, 0.0),
                       force=(1e-5, 0.0, 0.0), rho_solid=1.0,
                       face_type={"east": "periodic", "west": "periodic", "north": "noslip", "south": "noslip",
                                  "up": "noslip", "down": "noslip"},
                       face_vel={"up": (0.02, 0.0, 0.0), "down": (0.0, 0.0, 0.0), "north": (0.0, 0.0, 0.01),
                                 "south": (0.0, 0.0, 0.0)}),
    # D3Q19 periodic in y, moving walls east/west, open up/down (plbpd leaves
    # faces without an entry alone)
    "d3q19_ns_periodic": dict(model="D3Q19", nx=5, ny=6, nz=4, nu=0.2, rho0=1.0, u0=(0.0, 0.0, 0.0),
                              force=(1e-4, 2e-5, 0.0), rho_solid=1.0,
                              face_type={"north": "periodic", "south": "periodic", "east": "noslip",
                                         "west": "noslip"},
                              face_vel={"east": (0.0, 0.03, 0.0), "west": (0.0, 0.0, 0.0)}),
    # no boundary entries at all: every face open
    "d3q19_open": dict(model="D3Q19", nx=5, ny=4, nz=3, nu=0.3, rho0=1.0, u0=(0.02, -0.01, 0.005),
                       force=(0.0, 0.0, 0.0), rho_solid=1.0, face_type={}, face_vel={}),
    # thin domain: parallel walls only two layers apart interact
    "d3q19_thin_walls": dict(model="D3Q19", nx=4, ny=3, nz=3, nu=0.1, rho0=1.0, u0=(0.0, 0.0, 0.0),
                             force=(1e-4, 0.0, 0.0), rho_solid=1.0,
                             face_type={"east": "periodic", "west": "periodic", "north": "noslip",
                                        "south": "noslip", "up": "noslip", "down": "noslip"},
                             face_vel={"up": (0.01, 0.0, 0.0), "down": (0.0, 0.0, 0.0),
                                       "north": (0.0, 0.0, 0.02), "south": (0.0, 0.0, 0.0)}),
}

SOURCEMAP_CASES = {
    "d2q9_8x1x6": dict(model="D2Q9", nx=8, ny=1, nz=6, nu=0.1, rho0=1.0, u0=(0, 0, 0), force=(0, 0, 0),
                       rho_solid=1.0,
                       face_type={"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"},
                       face_vel={"up": (0, 0, 0), "down": (0, 0, 0)}),
    "d3q19_8x7x6_xy": dict(model="D3Q19", nx=8, ny=7, nz=6, nu=0.1, rho0=1.0, u0=(0, 0, 0), force=(0, 0, 0),
                           rho_solid=1.0,
                           face_type={"east": "periodic", "west": "periodic", "north": "periodic",
                                      "south": "periodic", "up": "noslip", "down": "noslip"},
                           face_vel={"up": (0, 0, 0), "down": (0, 0, 0)}),
    "d3q19_8x7x6_x": dict(model="D3Q19", nx=8, ny=7, nz=6, nu=0.1, rho0=1.0, u0=(0, 0, 0), force=(0, 0, 0),
                          rho_solid=1.0,
                          face_type={"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"},
                          face_vel={"up": (0, 0, 0), "down": (0, 0, 0)}),
    "d3q27_duct": dict(model="D3Q27", nx=6, ny=5, nz=7, nu=0.1, rho0=1.0, u0=(0, 0, 0), force=(0, 0, 0),
                       rho_solid=1.0,
                       face_type={"east": "periodic", "west": "periodic", "north": "noslip", "south": "noslip",
                                  "up": "noslip", "down": "noslip"},
                       face_vel={"up": (0, 0, 0), "down": (0, 0, 0), "north": (0, 0, 0), "south": (0, 0, 0)}),
}

# The small plain configuration: D2Q9 channel on a 128 x 64 lattice, tau = 0.8
# (nu = 0.1 gives 3*nu + 0.5 = 0.8 in float), periodic in x, resting walls on
# the first and last of the 64 layers, driven by the body force that gives a
# centre-line velocity of 0.01 at steady state: F = 8 nu u_max / H^2 with
# H = 62 (half-way walls) -> 2.08e-6.
CHANNEL = dict(model="D2Q9", nx=128, ny=1, nz=64, nu=0.1, rho0=1.0, u0=(0.0, 0.0, 0.0), force=(2.08e-6, 0.0, 0.0),
               rho_solid=1.0, face_type={"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"},
               face_vel={"up": (0.0, 0.0, 0.0), "down": (0.0, 0.0, 0.0)})

# plbpd's four Flow presets (src/Flow.cpp:20-106) with their step counts, as
# explicit configurations for the reference harness.
_XY = {"east": "periodic", "west": "periodic", "north": "periodic", "south": "periodic", "up": "noslip",
       "down": "noslip"}
_X = {"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"}
PRESETS = {
    "Couette2D": (dict(model="D2Q9", nx=100, ny=1, nz=25, nu=0.5, rho0=1.0, u0=(0, 0, 0), force=(0, 0, 0),
                       rho_solid=1.0, face_type=_X, face_vel={"up": (0.5, 0, 0), "down": (0, 0, 0)}), 20000),
    "Couette3D": (dict(model="D3Q19", nx=200, ny=50, nz=50, nu=0.5, rho0=1.0, u0=(0, 0, 0), force=(0, 0, 0),
                       rho_solid=1.0, face_type=_XY, face_vel={"up": (0.5, 0, 0), "down": (0, 0, 0)}), 200),
    "Poiseuille2D": (dict(model="D2Q9", nx=256, ny=1, nz=48, nu=0.1, rho0=1.0, u0=(0, 0, 0), force=(1e-5, 0, 0),
                          rho_solid=1.0, face_type=_X, face_vel={"up": (0, 0, 0), "down": (0, 0, 0)}), 5000),
    "Poiseuille3D": (dict(model="D3Q19", nx=256, ny=256, nz=48, nu=0.1, rho0=1.0, u0=(0, 0, 0), force=(1e-5, 0, 0),
                          rho_solid=1.0, face_type=_XY, face_vel={"up": (0, 0, 0), "down": (0, 0, 0)}), 10),
}
