"""Seeded synthetic workloads: scenes, RF setups and sensor poses.

World frame: y up. Antennas use the mounting of examples/src/1_dihedral.cpp:96-100
(`facing`, whose third column is the boresight) rotated about y.

  dihedral_workload      two 10 cm x 10 cm PEC plates at 90 degrees (4 triangles),
                         monostatic sensor at 1 m, azimuth 0..90 deg in 1 deg steps,
                         77-81 GHz, 256 ADC samples, 2 bounces, 2^18 samples per pose
  sphere_ground_workload icosphere level 6 (81,920 triangles, r = 0.5 m) on a 20 m x 20 m
                         ground quad, sensor at 10 m range and 0.5 m height, 3 bounces,
                         2^22 samples, 512 ADC samples at 10 MHz
  boxes_workload         ~1 M triangles of random axis-aligned boxes (edges 0.2-5 m) on a
                         100 m x 100 m ground quad, 4096 poses at 1 m height with random
                         yaw, log-uniform budgets 2^16..2^22, 4 bounces, 256 samples
"""
import dataclasses

import numpy as np

from .core import NFAntenna, TriangleMesh
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
