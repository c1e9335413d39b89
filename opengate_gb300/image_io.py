"""Minimal MetaImage (.mhd + .raw) reader and writer.

The reference reads CT images and writes actor outputs through ITK, whose
default format for this path is MetaImage (opengate/image.py, actor outputs
``*_edep.mhd`` etc.).  Only what the path needs is supported: 3D scalar
images, ElementType MET_SHORT / MET_USHORT / MET_UCHAR / MET_FLOAT /
MET_DOUBLE / MET_INT, little endian, a direction matrix (TransformMatrix,
the ITK direction cosines), raw data in a separate file (or LOCAL).  Arrays are returned in numpy [z][y][x] order as
ITK's GetArrayFromImage does; ``origin`` is the centre of the first voxel.
"""

import pathlib

import numpy as np

_TYPES = {
    "MET_CHAR": np.int8, "MET_UCHAR": np.uint8, "MET_SHORT": np.int16, "MET_USHORT": np.uint16,
    "MET_INT": np.int32, "MET_UINT": np.uint32, "MET_FLOAT": np.float32, "MET_DOUBLE": np.float64,
}
_NAMES = {np.dtype(v): k for k, v in _TYPES.items()}


class Image:
    """A 3D image: ``array`` [z][y][x], ``spacing`` and ``origin`` in mm (x, y, z)."""

    def __init__(self, array, spacing=(1.0, 1.0, 1.0), origin=None, direction=None):
        self.array = np.asarray(array)
        self.direction = np.eye(3) if direction is None else np.asarray(direction, dtype=np.float64).reshape(3, 3)
        if self.array.ndim != 3:
            raise ValueError("only 3D images are supported")
        self.spacing = np.asarray(spacing, dtype=np.float64)
        if origin is None:  # centred on (0, 0, 0), ITK half-voxel convention
            size = np.array(self.array.shape[::-1], dtype=np.float64)
            origin = -size * self.spacing / 2.0 + self.spacing / 2.0
        self.origin = np.asarray(origin, dtype=np.float64)

    @property
    def size(self):
        """(nx, ny, nz)."""
        return tuple(int(v) for v in self.array.shape[::-1])


def read_mhd(path):
    path = pathlib.Path(path)
    header = {}
    for line in path.read_text(errors="replace").splitlines():
        if "=" not in line:
            continue
        k, v = line.split("=", 1)
        header[k.strip()] = v.strip()
    if int(header.get("NDims", 3)) != 3:
        raise ValueError(f"{path}: only 3D MetaImages are supported")
    if header.get("BinaryDataByteOrderMSB", "False").lower() == "true" or \
            header.get("ElementByteOrderMSB", "False").lower() == "true":
        raise ValueError(f"{path}: big-endian data not supported")
    if int(header.get("ElementNumberOfChannels", 1)) != 1:
        raise ValueError(f"{path}: multi-channel images not supported")
    dims = [int(x) for x in header["DimSize"].split()]
    spacing = [float(x) for x in header.get("ElementSpacing", header.get("ElementSize", "1 1 1")).split()]
    origin = [float(x) for x in header.get("Offset", header.get("Origin", "0 0 0")).split()]
    dtype = _TYPES[header["ElementType"]]
    n = dims[0] * dims[1] * dims[2]
    df = header["ElementDataFile"]
    if df == "LOCAL":
        raw = path.read_bytes()
        data = np.frombuffer(raw[len(raw) - n * np.dtype(dtype).itemsize:], dtype=dtype)
    else:
        data = np.fromfile(path.parent / df, dtype=dtype, count=n)
    if data.size != n:
        raise ValueError(f"{path}: expected {n} elements, found {data.size}")
    tm = [float(x) for x in header.get("TransformMatrix", "1 0 0 0 1 0 0 0 1").split()]
    # MetaImage stores the direction column by column (ITK's writer)
    direction = np.array(tm, dtype=np.float64).reshape(3, 3).T
    return Image(data.reshape(dims[2], dims[1], dims[0]).copy(), spacing, origin, direction)


def write_mhd(path, image):
    path = pathlib.Path(path)
    if path.suffix != ".mhd":
        path = path.with_suffix(".mhd")
    arr = np.ascontiguousarray(image.array)
    if arr.dtype not in _NAMES:
        arr = arr.astype(np.float64)
    raw = path.with_suffix(".raw")
    nx, ny, nz = image.size
    lines = [
        "ObjectType = Image", "NDims = 3", "BinaryData = True", "BinaryDataByteOrderMSB = False",
        "CompressedData = False",
        "TransformMatrix = " + " ".join(repr(float(v)) for v in np.asarray(image.direction).T.ravel()),
        "Offset = " + " ".join(repr(float(v)) for v in image.origin), "CenterOfRotation = 0 0 0",
        "AnatomicalOrientation = RAI",
        "ElementSpacing = " + " ".join(repr(float(v)) for v in image.spacing),
        f"DimSize = {nx} {ny} {nz}", f"ElementType = {_NAMES[arr.dtype]}", f"ElementDataFile = {raw.name}",
    ]
    path.parent.mkdir(parents=True, exist_ok=True)
    path.write_text("\n".join(lines) + "\n")
    arr.tofile(raw)
    return path
