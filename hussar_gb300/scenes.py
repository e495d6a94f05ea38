"""Seeded synthetic workloads: scenes, RF setups and sensor poses.

World frame: y up. Antennas use the mounting of examples/src/1_dihedral.cpp:96-100
(`facing`, whose third column is the boresight) rotated about y.

  dihedral_workload      two 10 cm x 10 cm PEC plates at 90 degrees (4 triangles),
                         monostatic sensor at 1 m, azimuth 0..90 deg in 1 deg steps,
                         77-81 GHz, 256 ADC samples, 2 bounces, 2^18 samples per pose
  sphere_ground_workload icosphere level 6 (81,920 triangles, r = 0.5 m) on a 20 m x 20 m
                         ground quad, sensor at 10 m range and 0.5 m height, 3 bounces,
                         2^22 samples, 512 ADC samples at 10 MHz
  dihedral_ff_workload   the same dihedral lit and observed by far-field antennas (plane
                         waves, FFAntenna): monostatic, directions in the horizontal plane
                         from 5 to 85 deg azimuth, H along y, disk radius 0.1 m
  boxes_workload         ~1 M triangles of random axis-aligned boxes (edges 0.2-5 m) on a
                         100 m x 100 m ground quad, 4096 poses at 1 m height with random
                         yaw, log-uniform budgets 2^16..2^22, 4 bounces, 256 samples
"""
import dataclasses

import numpy as np

from .core import FFAntenna, NFAntenna, TriangleMesh
from .radar import FrameConfig, RFConfig

FACING = np.array([[0, 0, -1], [0, -1, 0], [-1, 0, 0]], np.float32)  # 1_dihedral.cpp:96-100


def rot_y(alpha):
    """Eigen::AngleAxisf(alpha, UnitY).toRotationMatrix()."""
    c, s = np.cos(alpha), np.sin(alpha)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], np.float64)


def looking(yaw):
    """Antenna rotation whose boresight is (-cos(yaw), 0, -sin(yaw))."""
    return (rot_y(-yaw) @ FACING.astype(np.float64)).astype(np.float32)


def rf_77ghz(samples=256, adc_rate=5e6):
    """77-81 GHz chirp: 4 GHz over 51.2 us (78.125 MHz/us), 0.43 ns antenna delay
    (1_dihedral.cpp:28), 100 us idle."""
    rf = RFConfig(startFreq=77e9, freqSlope=4e9 / 51.2e-6, adcRate=adc_rate, idleTime=100e-6, rampTime=51.2e-6,
                  antennaDelay=0.43e-9)
    return rf, FrameConfig(1, samples, 1)


def rf_chirp(bandwidth=4e9, samples=256, ramp=51.2e-6, start=77e9):
    """A chirp from `start` over `bandwidth` in `ramp` seconds, sampled `samples` times
    during the ramp (adcRate = samples / ramp), with rf_77ghz's delay and idle time."""
    return RFConfig(startFreq=start, freqSlope=bandwidth / ramp, adcRate=samples / ramp, idleTime=100e-6,
                    rampTime=ramp, antennaDelay=0.43e-9)


@dataclasses.dataclass
class Workload:
    name: str
    mesh: TriangleMesh
    rf: RFConfig
    frame: FrameConfig
    tx: list
    rx: list
    budget: np.ndarray
    max_depth: int


def dihedral_mesh(size=0.1):
    """Corner reflector: plate in x=0 (y,z in [0,size]) and plate in z=0 (x,y in [0,size])."""
    m = TriangleMesh()
    m.addQuad([0, 0, 0], [0, size, 0], [0, 0, size])
    m.addQuad([0, 0, 0], [size, 0, 0], [0, size, 0])
    return m


def dihedral_workload(poses=91, samples_per_pose=1 << 18, size=0.1, distance=1.0):
    mesh = dihedral_mesh(size)
    rf, fc = rf_77ghz(256, 5e6)
    tx, rx = [], []
    for k in range(poses):
        th = np.deg2rad(90.0 * k / max(poses - 1, 1))
        pos = np.array([distance * np.cos(th), size / 2, distance * np.sin(th)], np.float32)
        a = NFAntenna(pos, looking(th))
        tx.append(a)
        rx.append(a)
    return Workload("dihedral-4tri-91poses", mesh, rf, fc, tx, rx, np.full(poses, samples_per_pose, np.int64), 2)


def evaluation_dihedral_workload(size=0.05, angles_deg=None, samples_per_pose=1 << 19):
    """The reference's dihedral evaluation setup (examples/src/1_dihedral.cpp:24-109):
    two 2 mm thick plates (addBox) of edge `size` meeting at the y axis, an AWR sensor
    with TX at (896, 67, -7) mm and RX at (896, 67, -5) mm rotated about y by
    (angle - 45) degrees (Eigen::AngleAxisf, formed in float), facing the corner; chirp
    77 GHz + 60 MHz/us over 60 us, 5 MHz ADC, 256 samples, 0.43 ns antenna delay. The
    reference's evaluation data sweeps the angle over linspace(-75, 75, 601)."""
    mesh = TriangleMesh()
    mesh.addBox([-0.002, 0.0, 0.0], [0.0, size, size])
    mesh.addBox([0.0, 0.0, -0.002], [size, size, 0.0])
    rf = RFConfig(startFreq=77e9, freqSlope=60e6 / 1e-6, adcRate=5e6, idleTime=100e-6, rampTime=60e-6,
                  antennaDelay=0.43e-9)
    fc = FrameConfig(1, 256, 1)
    if angles_deg is None:
        angles_deg = np.linspace(-75.0, 75.0, 601)
    f32 = np.float32
    tx, rx = [], []
    for ang in angles_deg:
        a = (f32(ang) - f32(45)) / f32(180) * f32(np.pi)
        c, s = np.cos(a, dtype=np.float32), np.sin(a, dtype=np.float32)
        rot = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], np.float32)
        orient = (rot @ FACING).astype(np.float32)
        tx.append(NFAntenna((rot @ np.array([0.896, 0.067, -0.007], np.float32)).astype(np.float32), orient))
        rx.append(NFAntenna((rot @ np.array([0.896, 0.067, -0.005], np.float32)).astype(np.float32), orient))
    return Workload("evaluation-dihedral-%dmm" % round(size * 1000), mesh, rf, fc, tx, rx,
                    np.full(len(tx), samples_per_pose, np.int64), 10)


def dihedral_ff_workload(poses=9, samples_per_pose=1 << 16, size=0.1, radius=0.1):
    """Monostatic far-field sweep of the dihedral: TX = RX = FFAntenna with direction
    (cos a, 0, sin a), a = 5..85 deg (the corner opens towards +x+z), H = (0, 1, 0),
    scene centre the middle of the reflector's bounding cube."""
    mesh = dihedral_mesh(size)
    rf, fc = rf_77ghz(256, 5e6)
    center = np.array([size / 2, size / 2, size / 2], np.float32)
    tx = []
    for k in range(poses):
        a = np.deg2rad(5.0 + 80.0 * k / max(poses - 1, 1))
        d = np.array([np.cos(a), 0.0, np.sin(a)], np.float32)
        d /= np.float32(np.linalg.norm(d.astype(np.float64)))
        tx.append(FFAntenna(d, np.array([0, 1, 0], np.complex64), center, radius))
    return Workload("dihedral-ff-%dposes" % poses, mesh, rf, fc, tx, list(tx),
                    np.full(poses, samples_per_pose, np.int64), 2)


def icosphere(level, radius=1.0, center=(0, 0, 0)):
    """Icosahedron subdivided `level` times (20 * 4^level triangles), projected to the sphere."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(level):
        nv = len(v)
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], 0)
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid], 0)
        nf = len(f)
        a = nv + inv[:nf]
        b = nv + inv[nf:2 * nf]
        c = nv + inv[2 * nf:]
        f = np.concatenate([np.stack([f[:, 0], a, c], 1), np.stack([f[:, 1], b, a], 1),
                            np.stack([f[:, 2], c, b], 1), np.stack([a, b, c], 1)], 0)
    v = v * radius + np.asarray(center, np.float64)
    return v.astype(np.float32), f.astype(np.int32)


def sphere_ground_workload(samples=1 << 22, level=6):
    mesh = TriangleMesh()
    v, f = icosphere(level, 0.5, (0.0, 0.5, 0.0))
    mesh.append(v, f)
    mesh.addQuad([-10, 0, -10], [20, 0, 0], [0, 0, 20])
    rf, fc = rf_77ghz(512, 10e6)
    a = NFAntenna(np.array([10.0, 0.5, 0.0], np.float32), looking(0.0))
    return Workload("icosphere6+ground-81922tri", mesh, rf, fc, [a], [a], np.array([samples], np.int64), 3)


def boxes_mesh(seed=0xC3, count=83334, extent=100.0):
    """Random axis-aligned boxes (12 triangles each, mesh.h:42-54) on a ground quad."""
    rng = np.random.default_rng(seed)
    size = rng.uniform(0.2, 5.0, (count, 3))
    pos = rng.uniform(-extent / 2, extent / 2, (count, 2))
    mn = np.stack([pos[:, 0], np.zeros(count), pos[:, 1]], 1)
    mx = mn + size
    mn = mn.astype(np.float32)
    mx = mx.astype(np.float32)
    # vectorised addBox: 6 quads x 4 vertices per box, same vertex order as mesh.h:42-54
    d = mx - mn
    z = np.zeros(count, np.float32)

    def quad(a, b, c):
        ab = a + b
        return np.stack([a, ab, ab + c, a + c], 1)

    dx = np.stack([d[:, 0], z, z], 1)
    dy = np.stack([z, d[:, 1], z], 1)
    dz = np.stack([z, z, d[:, 2]], 1)
    quads = [quad(mn, dy, dz), quad(mn, dz, dx), quad(mn, dx, dy), quad(mx, -dy, -dx), quad(mx, -dz, -dy),
             quad(mx, -dx, -dz)]
    verts = np.stack(quads, 1).reshape(count * 24, 3).astype(np.float32)
    base = (np.arange(count * 6, dtype=np.int64) * 4)[:, None]
    tri = np.concatenate([base + np.array([0, 1, 2]), base + np.array([0, 2, 3])], 1).reshape(-1, 3)
    mesh = TriangleMesh()
    mesh.append(verts, tri.astype(np.int32))
    h = extent / 2
    mesh.addQuad([-h, 0, -h], [extent, 0, 0], [0, 0, extent])
    return mesh


def boxes_workload(poses=4096, seed=0xC3, count=83334, min_log2=16, max_log2=22):
    mesh = boxes_mesh(seed, count)
    rng = np.random.default_rng(seed + 1)
    rf, fc = rf_77ghz(256, 5e6)
    tx = []
    for _ in range(poses):
        x, z = rng.uniform(-50, 50, 2)
        yaw = rng.uniform(0, 2 * np.pi)
        tx.append(NFAntenna(np.array([x, 1.0, z], np.float32), looking(yaw)))
    budget = np.round(2.0 ** rng.uniform(min_log2, max_log2, poses)).astype(np.int64)
    return Workload("boxes-1Mtri-%dposes" % poses, mesh, rf, fc, tx, list(tx), budget, 4)


def _grid_quads(origin, u, v, nu, nv):
    """A parallelogram origin + [0,1]u + [0,1]v split into nu x nv quads (2 triangles
    each, addQuad's vertex order per cell). Returns (vertices, triangles)."""
    a = np.arange(nu + 1, dtype=np.float64) / nu
    b = np.arange(nv + 1, dtype=np.float64) / nv
    grid = origin[None, None, :] + a[:, None, None] * u[None, None, :] + b[None, :, None] * v[None, None, :]
    verts = grid.reshape(-1, 3)
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    p00 = (i * (nv + 1) + j).reshape(-1)
    p10 = p00 + (nv + 1)
    p11 = p10 + 1
    p01 = p00 + 1
    tri = np.concatenate([np.stack([p00, p10, p11], 1), np.stack([p00, p11, p01], 1)], 1).reshape(-1, 3)
    return verts, tri


def urban_mesh(target_tris=5_000_000, seed=0xC4, blocks=14, pitch=42.0, street=12.0, cars=200):
    """Synthetic urban canyon: a blocks x blocks grid of building boxes (footprint up to
    the block, height ~U(10, 40) m) separated by `street`-wide streets, walls and roofs
    tessellated into square cells sized so that the mesh has about `target_tris`
    triangles, plus `cars` 4.5 x 1.8 x 1.5 m boxes on the streets and a ground quad."""
    rng = np.random.default_rng(seed)
    block = pitch - street
    half = blocks * pitch / 2
    fx = rng.uniform(0.6, 1.0, (blocks, blocks)) * block
    fz = rng.uniform(0.6, 1.0, (blocks, blocks)) * block
    hh = rng.uniform(10.0, 40.0, (blocks, blocks))
    area = float(np.sum(2 * (fx + fz) * hh + fx * fz))
    budget = max(target_tris - 12 * cars - 2, 1000)
    cell = np.sqrt(2.0 * area / budget)
    vs, ts, nv = [], [], 0
    for bi in range(blocks):
        for bj in range(blocks):
            x0 = -half + bi * pitch + street / 2
            z0 = -half + bj * pitch + street / 2
            mn = np.array([x0, 0.0, z0])
            mx = mn + np.array([fx[bi, bj], hh[bi, bj], fz[bi, bj]])
            d = mx - mn
            ex, ey, ez = np.array([d[0], 0, 0]), np.array([0, d[1], 0]), np.array([0, 0, d[2]])
            n = lambda L: max(1, int(round(L / cell)))
            faces = [(mn, ex, ey), (mn, ez, ey), (mn + ez, ex, ey), (mn + ex, ez, ey), (mn + ey, ex, ez)]
            for o, u, v in faces:
                gv, gt = _grid_quads(o, u, v, n(np.linalg.norm(u)), n(np.linalg.norm(v)))
                vs.append(gv)
                ts.append(gt + nv)
                nv += len(gv)
    mesh = TriangleMesh()
    mesh.append(np.concatenate(vs).astype(np.float32), np.concatenate(ts).astype(np.int32))
    # cars on the street lines, parallel to the street
    for _ in range(cars):
        along = rng.uniform(-half, half)
        line = -half + int(rng.integers(0, blocks + 1)) * pitch
        side = rng.choice([-3.0, 3.0])
        if rng.random() < 0.5:
            mn = np.array([along, 0.0, line + side - 0.9])
            mx = mn + np.array([4.5, 1.5, 1.8])
        else:
            mn = np.array([line + side - 0.9, 0.0, along])
            mx = mn + np.array([1.8, 1.5, 4.5])
        mesh.addBox(mn.astype(np.float32), mx.astype(np.float32))
    mesh.addQuad([-half, 0, -half], [2 * half, 0, 0], [0, 0, 2 * half])
    return mesh


def street_poses(count, seed, blocks=14, pitch=42.0, height=1.0):
    """Sensors on the street centre lines of urban_mesh at `height`, random yaw."""
    rng = np.random.default_rng(seed)
    half = blocks * pitch / 2
    out = []
    for _ in range(count):
        along = rng.uniform(-half, half)
        line = -half + int(rng.integers(0, blocks + 1)) * pitch
        x, z = (along, line) if rng.random() < 0.5 else (line, along)
        out.append(NFAntenna(np.array([x, height, z], np.float32), looking(rng.uniform(0, 2 * np.pi))))
    return out


def plane_poses(count, seed, extent=100.0, height=1.0):
    """Sensors uniform over the boxes ground quad at `height`, random yaw."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        x, z = rng.uniform(-extent / 2, extent / 2, 2)
        out.append(NFAntenna(np.array([x, height, z], np.float32), looking(rng.uniform(0, 2 * np.pi))))
    return out


# Resident scenes of the serving workload: the boxes generator at the batched workload's
# density (extent grows with the box count) and the urban-canyon generator, alternating,
# at 100 k .. 5 M triangles.
SERVE_SCENES = [("boxes", 100_000), ("urban", 250_000), ("boxes", 500_000), ("urban", 1_000_000),
                ("boxes", 2_000_000), ("urban", 3_000_000), ("boxes", 4_000_000), ("urban", 5_000_000)]


def serve_scene(kind, tris, seed):
    """(mesh, pose generator) of one resident serving scene."""
    if kind == "boxes":
        count = max(1, (tris - 2) // 12)
        extent = 100.0 * np.sqrt(count / 83334.0)
        return boxes_mesh(seed, count, extent), (lambda n, s: plane_poses(n, s, extent))
    return urban_mesh(tris, seed), (lambda n, s: street_poses(n, s))


def mimo_array(position, yaw, n_tx=3, n_rx=4, start_freq=77e9):
    """TX and RX antennas of a MIMO radar at `position` looking along `yaw`: RX elements
    half a wavelength (at `start_freq`) apart along the array's horizontal axis, TX
    elements n_rx half-wavelengths apart, so the n_tx x n_rx (TX, RX) pairs form a
    uniform virtual array of half-wavelength spacing. Returns (tx list, rx list)."""
    half = 299792458.0 / start_freq / 2.0
    R = looking(yaw).astype(np.float64)
    axis = R[:, 0]  # horizontal, perpendicular to the boresight R[:, 2]
    p = np.asarray(position, np.float64)
    tx = [NFAntenna((p + axis * (i * n_rx * half)).astype(np.float32), R.astype(np.float32)) for i in range(n_tx)]
    rx = [NFAntenna((p + axis * (j * half)).astype(np.float32), R.astype(np.float32)) for j in range(n_rx)]
    return tx, rx


def urban_mimo_workload(tris=5_000_000, seed=0xC4, samples=1 << 22, chirps=128):
    """The guided urban MIMO configuration: the urban canyon (about `tris` triangles),
    one sensor on a street at 1 m with a 3 TX x 4 RX array at half-wavelength spacing
    (12 virtual channels, each a (TX, RX) pose of one batch), 77-81 GHz, 256 samples per
    chirp, `chirps` chirps per frame, up to 5 bounces; `samples` per channel."""
    mesh = urban_mesh(tris, seed)
    rng = np.random.default_rng(seed + 7)
    pose = street_poses(1, seed + 9)[0]
    yaw = float(rng.uniform(0, 2 * np.pi))
    txs, rxs = mimo_array(pose.position(), yaw)
    tx = [t for t in txs for _ in rxs]
    rx = [r for _ in txs for r in rxs]
    rf, _ = rf_77ghz(256)
    fc = FrameConfig(chirps, 256, len(tx))
    w = Workload("urban-%dk-mimo3x4" % (tris // 1000), mesh, rf, fc, tx, rx, np.full(len(tx), samples, np.int64), 5)
    w.tx_array, w.rx_array = txs, rxs  # the physical array (hsr_simulate_frame's arguments)
    return w
