"""Scene input and frame output in the reference's formats.

WavefrontFile   hussar::WavefrontFile (libhussar/include/hussar/io/wavefront.h:12-67):
                OBJ vertices and triangles appended to a TriangleMesh.
write_frame     writeFrameToFile (examples/src/utils.h:29-35): a frame's samples in
                index order, each as two floats (re, im); the examples append one frame
                per pose to one file (examples/src/1_dihedral.cpp:87-126).
save_frame      saveFrame (utils.h:37-40): one frame to `<path>.SIM`.
read_sim        the inverse: every frame of a .SIM file as complex64 cubes.
"""
import numpy as np

from .radar import Frame


class WavefrontFile:
    """hussar::WavefrontFile: read(mesh) appends the file's vertices and triangles.

    Line by line, as the reference parses them: a line starting with '#' is a comment;
    'v x y z' adds a vertex (further components are ignored); 'f a b c' adds a triangle
    from the first three 1-based vertex indices, counted from the vertices the mesh had
    before this read (further indices on the line are ignored); 's' and empty lines are
    skipped; any other command is reported and skipped. The reference reads the index
    tokens with `>> int`, so 'a/b/c' tokens stop its stream; here the vertex index before
    the first '/' is taken instead."""

    def __init__(self, path):
        self.path = path
        self.unsupported = []  # commands the reader skipped, in order

    def read(self, mesh):
        try:
            fh = open(self.path, "r")
        except OSError:
            raise ValueError("invalid file passed to WavefrontFile: %s" % self.path)
        offset = mesh.vertexBuffer.shape[0]  # wavefront.h:23: vertices already in the mesh
        verts, tris = [], []
        with fh:
            for line in fh:
                if line.startswith("#"):
                    continue
                tok = line.split()
                if not tok:
                    continue
                cmd = tok[0]
                if cmd == "v":
                    verts.append([np.float32(float(t)) for t in tok[1:4]])
                elif cmd == "f":
                    tris.append([int(t.split("/")[0]) + offset - 1 for t in tok[1:4]])
                elif cmd == "s":
                    pass
                else:
                    self.unsupported.append(cmd)
        v = np.array(verts, np.float32).reshape(-1, 3)
        f = np.array(tris, np.int64).reshape(-1, 3)
        # TriangleMesh.append takes indices relative to the appended vertices
        mesh.append(v, (f - offset).astype(np.int32))
        return mesh


def write_frame(fh, frame):
    """writeFrameToFile: the frame's samples as (re, im) float pairs, index order."""
    data = frame.data if isinstance(frame, Frame) else np.asarray(frame)
    fh.write(np.ascontiguousarray(data, np.complex64).tobytes())
    fh.flush()


def save_frame(frame, path):
    """saveFrame: one frame to `path + '.SIM'`."""
    with open(path + ".SIM", "wb") as fh:
        write_frame(fh, frame)


def read_sim(path, config):
    """Frames of a .SIM file as complex64 cubes [frames, chirps, samples, channels]."""
    raw = np.fromfile(path, np.complex64)
    n = config.sampleCount()
    if n == 0 or raw.size % n:
        raise ValueError("file size is not a whole number of %d-sample frames" % n)
    return raw.reshape(-1, config.chirpCount, config.samplesPerChirp, config.channelCount)
