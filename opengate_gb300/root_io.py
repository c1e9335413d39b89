"""ROOT files with one flat TTree: the on-disk format of the reference's digi collections.

The reference writes each digi collection (hits, singles, the energy windows'
channels) as a Geant4 ntuple in a ROOT file, one row per digi and one column
per attribute (GateDigiCollection::FillToRoot,
core/opengate_core/opengate_lib/digitizer/GateDigiCollection.cpp:114-128,
through GateDigiCollectionsRootManager and Geant4's ROOT writer; a 3-vector
attribute becomes three columns ``<name>_X/_Y/_Z``).  This module writes the
same layout without ROOT installed: a file of ROOT's small-file format
(32-bit seeks) holding one uncompressed TTree whose branches each carry one
leaf of a fixed-size type (``D`` double, ``F`` float, ``I`` int32, ``L``
int64, unsigned variants flagged on the leaf), stored in baskets of at most
``basket_entries`` entries.  ``read_tree`` reads such files back (the
round-trip check; it understands what ``write_tree`` writes, not ROOT files
in general).

Layout written (big-endian, as ROOT): file header at 0; the top directory
record at 100; the baskets; the TTree key; an empty StreamerInfo list (the
classes are written at the versions ROOT's own dictionaries hold: TTree 20,
TBranch 13, TLeaf 2, TLeaf[DFIL] 1, TObjArray 3, TNamed 1); the key list;
the free-segment record.
"""

import struct
import time

import numpy as np

_K_BYTECOUNT = 0x40000000
_K_NEW_CLASS = 0xFFFFFFFF
_K_CLASS_MASK = 0x80000000
_K_MAP_OFFSET = 2
_BEGIN = 100
_FILE_VERSION = 62206  # a small-file (32-bit seek) version number
_OBJ_BITS = 0x03000000  # kNotDeleted | kIsOnHeap, as ROOT stores them

# leaf code -> (leaf class, numpy big-endian dtype, unsigned)
_LEAVES = {
    "D": ("TLeafD", ">f8", False), "F": ("TLeafF", ">f4", False),
    "I": ("TLeafI", ">i4", False), "i": ("TLeafI", ">u4", True),
    "L": ("TLeafL", ">i8", False), "l": ("TLeafL", ">u8", True),
}
_CODE_OF = {np.dtype(np.float64): "D", np.dtype(np.float32): "F", np.dtype(np.int32): "I",
            np.dtype(np.uint32): "i", np.dtype(np.int64): "L", np.dtype(np.uint64): "l"}


def _datime(t=None):
    tm = time.gmtime(t)
    return ((tm.tm_year - 1995) << 26 | tm.tm_mon << 22 | tm.tm_mday << 17 | tm.tm_hour << 12 | tm.tm_min << 6
            | tm.tm_sec)


def _tstring(s):
    b = s.encode()
    if len(b) < 255:
        return bytes([len(b)]) + b
    return b"\xff" + struct.pack(">i", len(b)) + b


class _Buf:
    """Object buffer of one key: offsets count from the key's first byte (the reference
    tags of ROOT's object map), so the key header length is the buffer's origin."""

    def __init__(self, origin):
        self.b = bytearray()
        self.origin = origin
        self.classes = {}
        self.objects = {}

    def pos(self):
        return self.origin + len(self.b)

    def put(self, fmt, *v):
        self.b += struct.pack(">" + fmt, *v)

    def raw(self, data):
        self.b += data

    def begin(self, version):
        """Byte count placeholder + version; returns the placeholder's index."""
        at = len(self.b)
        self.put("Ih", 0, version)
        return at

    def end(self, at):
        struct.pack_into(">I", self.b, at, (len(self.b) - at - 4) | _K_BYTECOUNT)

    def tobject(self):
        self.put("hII", 1, 0, _OBJ_BITS)

    def tnamed(self, name, title):
        at = self.begin(1)
        self.tobject()
        self.raw(_tstring(name) + _tstring(title))
        self.end(at)

    def object(self, cls, key, write):
        """A pointer member: new object (byte count, class tag, body) or a reference."""
        if key is None:
            self.put("I", 0)
            return
        if key in self.objects:
            self.put("I", self.objects[key])
            return
        at = len(self.b)
        self.objects[key] = self.pos() + _K_MAP_OFFSET
        self.put("I", 0)
        if cls in self.classes:
            self.put("I", self.classes[cls] | _K_CLASS_MASK)
        else:
            self.classes[cls] = self.pos() + _K_MAP_OFFSET
            self.put("I", _K_NEW_CLASS)
            self.raw(cls.encode() + b"\0")
        write()
        self.end(at)

    def objarray(self, items):
        """TObjArray (v3) of (class, key, writer) entries."""
        at = self.begin(3)
        self.tobject()
        self.raw(_tstring(""))
        self.put("ii", len(items), 0)
        for cls, key, write in items:
            self.object(cls, key, write)
        self.end(at)

    def att(self, version, fmt, *v):
        at = self.begin(version)
        self.put(fmt, *v)
        self.end(at)

    def io_features(self):
        at = self.begin(1)
        self.put("B", 0)
        self.end(at)

    def counted_array(self, fmt, values):
        """A [count] pointer member: presence byte, then the elements."""
        self.put("b", 1 if len(values) else 0)
        for v in values:
            self.put(fmt, v)


def _key_header(nbytes, objlen, keylen, seek, pdir, cls, name, title, datime):
    return (struct.pack(">ihiIhhii", nbytes, 4, objlen, datime, keylen, 1, seek, pdir)
            + _tstring(cls) + _tstring(name) + _tstring(title))


def _keylen(cls, name, title):
    return 26 + len(_tstring(cls)) + len(_tstring(name)) + len(_tstring(title))


def write_tree(path, tree_name, columns, title=None, basket_entries=32000):
    """Writes `columns` ({branch name: 1-D array}, equal lengths; float64, float32, int32,
    uint32, int64 or uint64) as TTree `tree_name` in a new ROOT file at `path`."""
    title = tree_name if title is None else title
    names = list(columns)
    if not names:
        raise ValueError("a tree needs at least one column")
    arrays = {}
    for n in names:
        a = np.asarray(columns[n])
        if a.ndim != 1:
            raise ValueError(f"column {n}: one value per entry")
        if a.dtype not in _CODE_OF:
            raise ValueError(f"column {n}: dtype {a.dtype} has no fixed-size ROOT leaf here")
        arrays[n] = a
    n_entries = len(arrays[names[0]])
    if any(len(a) != n_entries for a in arrays.values()):
        raise ValueError("columns of different lengths")
    if basket_entries < 1:
        raise ValueError("basket_entries >= 1")
    fname = str(path).rsplit("/", 1)[-1]
    now = _datime()
    out = bytearray(_BEGIN)
    # ---- top directory record (rewritten once the seeks are known) -------------
    top_key_len = _keylen("TFile", fname, "")
    named = _tstring(fname) + _tstring("")
    dir_len = 2 + 4 * 7 + 18 + 12
    top_objlen = len(named) + dir_len
    out += b"\0" * (top_key_len + top_objlen)
    # ---- baskets ---------------------------------------------------------------
    branch_info = {}
    for n in names:
        code = _CODE_OF[arrays[n].dtype]
        dt = np.dtype(_LEAVES[code][1])
        data = arrays[n].astype(dt, copy=False)
        seeks, nbytes, firsts = [], [], []
        for first in range(0, n_entries, basket_entries):
            chunk = data[first:first + basket_entries].tobytes()
            cnt = min(basket_entries, n_entries - first)
            klen = _keylen("TBasket", n, tree_name) + 19
            seek = len(out)
            hdr = _key_header(klen + len(chunk), len(chunk), klen, seek, _BEGIN, "TBasket", n, tree_name, now)
            hdr += struct.pack(">hiiiib", 3, 32000, dt.itemsize, cnt, klen + len(chunk), 0)
            assert len(hdr) == klen
            out += hdr + chunk
            seeks.append(seek)
            nbytes.append(klen + len(chunk))
            firsts.append(first)
        branch_info[n] = (code, seeks, nbytes, firsts)
    # ---- the TTree key -----------------------------------------------------------
    tree_seek = len(out)
    tree_klen = _keylen("TTree", tree_name, title)
    buf = _Buf(tree_klen)
    tot = sum(sum(v[2]) for v in branch_info.values())
    at = buf.begin(20)
    buf.tnamed(tree_name, title)
    buf.att(2, "hhh", 602, 1, 1)  # TAttLine
    buf.att(2, "hh", 0, 1001)     # TAttFill
    buf.att(2, "hhf", 1, 1, 1.0)  # TAttMarker
    buf.put("qqqqqdiiiiiqqqqqq", n_entries, tot, tot, tot, 0, 1.0, 0, 25, 0, 0, 0,
            1000000000000, 1000000000000, 0, -300000000, -30000000, 1000000)
    buf.counted_array("q", [])  # fClusterRangeEnd
    buf.counted_array("q", [])  # fClusterSize
    buf.io_features()

    def leaf_writer(n):
        cls, dt, unsigned = _LEAVES[branch_info[n][0]]
        size = np.dtype(dt).itemsize

        def w():
            lat = buf.begin(1)
            tat = buf.begin(2)  # TLeaf
            buf.tnamed(n, n)
            buf.put("iii??I", 1, size, 0, False, unsigned, 0)
            buf.end(tat)
            vals = arrays[n]
            lo, hi = (vals.min(), vals.max()) if len(vals) else (0, 0)
            if cls in ("TLeafD", "TLeafF"):
                buf.put("dd" if cls == "TLeafD" else "ff", float(lo), float(hi))
            else:  # the extremes as the leaf's signed type (an unsigned leaf keeps the bit pattern)
                sdt = ">i8" if size == 8 else ">i4"
                ext = np.array([lo, hi]).astype(dt).view(sdt)
                buf.put("qq" if size == 8 else "ii", int(ext[0]), int(ext[1]))
            buf.end(lat)
        return w

    def branch_writer(n):
        code, seeks, nbytes, firsts = branch_info[n]
        nb = len(seeks)
        max_baskets = max(10, nb + 1)

        def w():
            bat = buf.begin(13)
            buf.tnamed(n, f"{n}/{code}")
            buf.att(2, "hh", 0, 1001)  # TAttFill
            buf.put("iiiiq", 0, 32000, 0, nb, n_entries)  # fCompress, fBasketSize, fEntryOffsetLen, fWriteBasket
            buf.io_features()
            buf.put("iiiqqqq", 0, max_baskets, 0, n_entries, 0, sum(nbytes), sum(nbytes))
            buf.objarray([])  # fBranches
            buf.objarray([(_LEAVES[code][0], ("leaf", n), leaf_writer(n))])
            buf.objarray([])  # fBaskets: every basket is on disk
            pad = max_baskets - nb
            buf.counted_array("i", nbytes + [0] * pad)
            buf.counted_array("q", firsts + [n_entries] + [0] * (pad - 1))
            buf.counted_array("q", seeks + [0] * pad)
            buf.raw(_tstring(""))  # fFileName
            buf.end(bat)
        return w

    buf.objarray([("TBranch", ("branch", n), branch_writer(n)) for n in names])
    buf.objarray([(_LEAVES[branch_info[n][0]][0], ("leaf", n), leaf_writer(n)) for n in names])
    buf.put("I", 0)                         # fAliases
    buf.put("i", 0)                         # fIndexValues (TArrayD, empty)
    buf.put("i", 0)                         # fIndex (TArrayI, empty)
    buf.put("IIII", 0, 0, 0, 0)             # fTreeIndex, fFriends, fUserInfo, fBranchRef
    buf.end(at)
    body = bytes(buf.b)
    out += _key_header(tree_klen + len(body), len(body), tree_klen, tree_seek, _BEGIN, "TTree", tree_name, title,
                       now) + body
    keys = [_key_header(tree_klen + len(body), len(body), tree_klen, tree_seek, _BEGIN, "TTree", tree_name, title,
                        now)]
    # ---- StreamerInfo (empty TList) ---------------------------------------------
    info_seek = len(out)
    info_klen = _keylen("TList", "StreamerInfo", "Doubly linked list")
    ib = _Buf(info_klen)
    iat = ib.begin(5)
    ib.tobject()
    ib.raw(_tstring(""))
    ib.put("i", 0)
    ib.end(iat)
    info = bytes(ib.b)
    info_nbytes = info_klen + len(info)
    out += _key_header(info_nbytes, len(info), info_klen, info_seek, _BEGIN, "TList", "StreamerInfo",
                       "Doubly linked list", now) + info
    # ---- key list ------------------------------------------------------------------
    keys_seek = len(out)
    kl_klen = _keylen("TFile", fname, "")
    kbody = struct.pack(">i", len(keys)) + b"".join(keys)
    keys_nbytes = kl_klen + len(kbody)
    out += _key_header(keys_nbytes, len(kbody), kl_klen, keys_seek, _BEGIN, "TFile", fname, "", now) + kbody
    # ---- free segments -------------------------------------------------------------
    free_seek = len(out)
    fr_klen = _keylen("TFile", fname, "")
    free_nbytes = fr_klen + 10
    end = free_seek + free_nbytes
    fbody = struct.pack(">hii", 1, end, 2000000000)
    out += _key_header(free_nbytes, len(fbody), fr_klen, free_seek, _BEGIN, "TFile", fname, "", now) + fbody
    assert len(out) == end
    # ---- top directory and file header --------------------------------------------
    uuid = struct.pack(">h", 1) + bytes(16)
    nbytes_name = top_key_len + len(named)
    top = (_key_header(top_key_len + top_objlen, top_objlen, top_key_len, _BEGIN, 0, "TFile", fname, "", now)
           + named + struct.pack(">hIIiiiii", 5, now, now, keys_nbytes, nbytes_name, _BEGIN, 0, keys_seek)
           + uuid + bytes(12))
    out[_BEGIN:_BEGIN + len(top)] = top
    hdr = (b"root" + struct.pack(">iiiiiiiBiii", _FILE_VERSION, _BEGIN, end, free_seek, free_nbytes, 1, nbytes_name,
                                 4, 0, info_seek, info_nbytes) + uuid)
    out[:len(hdr)] = hdr
    with open(path, "wb") as f:
        f.write(out)


def read_tree(path, tree_name):
    """Columns {branch: numpy array} of a TTree written by write_tree."""
    data = open(path, "rb").read()
    if data[:4] != b"root":
        raise ValueError(f"{path}: not a ROOT file")
    version, begin = struct.unpack_from(">ii", data, 4)
    if version >= 1000000:
        raise ValueError("large-file (64-bit seek) layout is not read here")

    def tstr(at):
        n = data[at]
        if n == 255:
            n = struct.unpack_from(">i", data, at + 1)[0]
            return data[at + 5:at + 5 + n].decode(), at + 5 + n
        return data[at + 1:at + 1 + n].decode(), at + 1 + n

    def key(at):
        nbytes, _, objlen, _, keylen, _, seek, _ = struct.unpack_from(">ihiIhhii", data, at)
        cls, p = tstr(at + 26)
        name, p = tstr(p)
        title, p = tstr(p)
        return dict(nbytes=nbytes, objlen=objlen, keylen=keylen, seek=seek, cls=cls, name=name, title=title, end=p)

    top = key(begin)
    _, p = tstr(top["end"])
    _, p = tstr(p)
    seek_keys = struct.unpack_from(">hIIiiiii", data, p)[7]
    kl = key(seek_keys)
    nkeys = struct.unpack_from(">i", data, seek_keys + kl["keylen"])[0]
    p = seek_keys + kl["keylen"] + 4
    tree = None
    for _ in range(nkeys):
        k = key(p)
        if k["cls"] == "TTree" and k["name"] == tree_name:
            tree = k
        p = k["end"]
    if tree is None:
        raise KeyError(f"{path}: no TTree {tree_name}")
    # the tree body, member by member in the order write_tree streams it
    t0 = tree["seek"]
    cur = _Cursor(data, t0 + tree["keylen"])
    cur.version(20)
    cur.tnamed()
    for v in (2, 2, 2):  # TAttLine, TAttFill, TAttMarker
        cur.skip_versioned(v)
    n_entries = cur.get("q")
    cur.get("qqqqdiiiiiqqqqqq")
    for _ in range(2):  # fClusterRangeEnd, fClusterSize (empty)
        if cur.get("b"):
            raise ValueError(f"{path}: cluster ranges are not read here")
    cur.skip_versioned(1)  # fIOFeatures
    out = {}
    for _ in range(cur.objarray()):
        cur.object_header("TBranch")
        cur.version(13)
        name, btitle = cur.tnamed()
        code = btitle.rsplit("/", 1)[-1]
        if code not in _LEAVES:
            raise ValueError(f"{path}: branch {name}: leaf type {code}")
        cur.skip_versioned(2)  # TAttFill
        _, _, _, n_baskets, _ = cur.get("iiiiq")
        cur.skip_versioned(1)
        _, max_baskets, _, b_entries, _, _, _ = cur.get("iiiqqqq")
        if cur.objarray():
            raise ValueError(f"{path}: sub-branches are not read here")
        for _ in range(cur.objarray()):  # the branch's leaf
            cur.object_header(_LEAVES[code][0])
            cur.skip_rest()
        if cur.objarray():
            raise ValueError(f"{path}: baskets kept in the tree are not read here")
        arrays = [cur.counted(f, max_baskets) for f in "iqq"]
        if any(len(a) != max_baskets for a in arrays):
            raise ValueError(f"{path}: branch {name}: basket arrays")
        dt = np.dtype(_LEAVES[code][1])
        vals = []
        for b in range(n_baskets):
            k = key(arrays[2][b])
            if k["cls"] != "TBasket" or k["name"] != name or k["nbytes"] != arrays[0][b]:
                raise ValueError(f"{path}: branch {name}: basket {b} not where the tree says")
            _, _, nevsize, nev, _, _ = struct.unpack_from(">hiiiib", data, k["end"])
            if nevsize != dt.itemsize or nev != arrays[1][b + 1] - arrays[1][b]:
                raise ValueError(f"{path}: branch {name}: basket {b} entries")
            vals.append(np.frombuffer(data, dtype=dt, count=nev, offset=arrays[2][b] + k["keylen"]))
        a = np.concatenate(vals) if vals else np.zeros(0, dt)
        if len(a) != b_entries or len(a) != n_entries:
            raise ValueError(f"{path}: branch {name} holds {len(a)} entries, the tree {n_entries}")
        out[name] = a.astype(dt.newbyteorder("="))
        cur.tstring()  # fFileName
        cur.close_object()
    return out


class _Cursor:
    """Sequential reader of a streamed object body (byte counts checked on close)."""

    def __init__(self, data, at):
        self.d = data
        self.p = at
        self.ends = []

    def get(self, fmt):
        v = struct.unpack_from(">" + fmt, self.d, self.p)
        self.p += struct.calcsize(">" + fmt)
        return v[0] if len(v) == 1 else v

    def version(self, want):
        cnt, v = self.get("Ih")
        if not cnt & _K_BYTECOUNT or v != want:
            raise ValueError(f"unexpected class version {v} (want {want})")
        return cnt

    def skip_versioned(self, want):
        cnt = self.version(want)
        self.p += (cnt & ~_K_BYTECOUNT) - 2

    def tstring(self):
        n = self.get("B")
        if n == 255:
            n = self.get("i")
        s = self.d[self.p:self.p + n].decode()
        self.p += n
        return s

    def tnamed(self):
        self.version(1)
        self.get("hII")
        return self.tstring(), self.tstring()

    def objarray(self):
        self.version(3)
        self.get("hII")
        self.tstring()
        n, _ = self.get("ii")
        return n

    def object_header(self, cls):
        start = self.p
        cnt = self.get("I")
        tag = self.get("I")
        if tag == _K_NEW_CLASS:
            end = self.d.index(b"\0", self.p)
            name = self.d[self.p:end].decode()
            self.p = end + 1
            if name != cls:
                raise ValueError(f"object of class {name}, expected {cls}")
        elif not tag & _K_CLASS_MASK:
            raise ValueError("object reference where an object was expected")
        self.ends.append(start + 4 + (cnt & ~_K_BYTECOUNT))

    def skip_rest(self):
        self.p = self.ends.pop()

    def close_object(self):
        end = self.ends.pop()
        if self.p != end:
            raise ValueError("object body length differs from its byte count")

    def counted(self, fmt, n):
        if not self.get("b"):
            return []
        v = struct.unpack_from(f">{n}{fmt}", self.d, self.p)
        self.p += struct.calcsize(f">{n}{fmt}")
        return list(v)
