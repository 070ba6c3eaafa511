"""Camera matrices and image output for the deferred point-splat renderer
(iso_point_splat_render), after examples/deferred_rasterisation.rs:223-236.

Matrices are 4 x 4, column-major float32 (element (row, col) at [col * 4 +
row]), computed here in double precision from cgmath's formulas
(`perspective`, `Matrix4::look_at`, right-handed).
"""
import numpy as np

# the example's settings (examples/deferred_rasterisation.rs:59-76, 223-236, 396-400)
FOVY_DEG = 45.0
NEAR, FAR = 0.01, 1000.0
EYE, CENTRE, UP = (-0.25, -0.25, -0.25), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0)
CLEAR_RGB = (0.306, 0.267, 0.698)


def perspective(fovy_deg, aspect, near, far):
    f = 1.0 / np.tan(np.radians(fovy_deg) / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = (far + near) / (near - far)
    m[3, 2] = -1.0
    m[2, 3] = 2.0 * far * near / (near - far)
    return m


def look_at(eye, centre, up):
    eye, centre, up = (np.asarray(v, np.float64) for v in (eye, centre, up))
    f = centre - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def column_major(m):
    return np.ascontiguousarray(np.asarray(m, np.float64).T.reshape(16).astype(np.float32))


def splat_camera(width, height):
    """(view_projection, its inverse) of the example's camera for an image of
    width x height pixels, column-major float32 (the model matrix is the
    identity)."""
    vp = perspective(FOVY_DEG, width / height, NEAR, FAR) @ look_at(EYE, CENTRE, UP)
    return column_major(vp), column_major(np.linalg.inv(vp))


def write_ppm(path, rgba):
    """Write an (h, w, 4) float image whose row 0 is the bottom row (the
    renderer's convention) as a binary PPM, top row first."""
    rgb = np.clip(np.asarray(rgba)[::-1, :, :3], 0.0, 1.0)
    data = (rgb * 255.0 + 0.5).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (data.shape[1], data.shape[0]))
        f.write(data.tobytes())
