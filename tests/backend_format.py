"""Writers for the reference's on-disk inputs, used to build test fixtures:

* the backend column store of RasterJoin/db (HashGridIndex.cpp:12-33,
  PartitioningManager.cpp:36-99, BufferedPartitionedFile.cpp:135-200):
  ``<stem>_config`` (QDataStream, big-endian: lx, ly as doubles, lz uint32,
  p1 p2 p3 int32, attribute count and types as quint8) and per attribute
  ``<stem><id>_payload.dat`` (raw little-endian values, partition chunks
  back to back) with ``<stem><id>_mapping`` (QHash<qint64,
  QVector<QPair<quint64, quint64>>>: quint32 count, then key, quint32 chunk
  count, (offset, size) pairs);
* the polygon text format ``tot {np {n x y ...}}`` (PolyHandler.cpp:133-188)
  and the collection list ``name,file`` (PolyHandler.cpp:20-40).
"""
import struct

import numpy as np

P1, P2, P3 = 73856093, 19349663, 83492791


def partition_ids(x, y, t, lx, ly, lz):
    """HashGridIndex::getPartitionId (HashGridIndex.cpp:98-113) per record."""
    xo = (np.asarray(x, np.float32) / np.float32(lx)).astype(np.int64)
    yo = (np.asarray(y, np.float32) / np.float32(ly)).astype(np.int64)
    zo = (np.asarray(t, np.uint32) // np.uint32(lz)).astype(np.int64)
    return (xo * P1) ^ (yo * P2) ^ (zo * P3)


def region_partitions(lo, hi, lx, ly, lz):
    """HashGridIndex::getIntersectingPartitions (HashGridIndex.cpp:117-141)."""
    f = np.float32
    x0, y0, z0 = int(f(lo[0]) / f(lx)), int(f(lo[1]) / f(ly)), int(f(lo[2]) / f(lz))
    x1, y1, z1 = int(f(hi[0]) / f(lx)), int(f(hi[1]) / f(ly)), int(f(hi[2]) / f(lz))
    out = set()
    for x in range(x0, x1 + 1):
        for y in range(y0, y1 + 1):
            for z in range(z0, z1 + 1):
                out.add(np.int64(x * P1) ^ np.int64(y * P2) ^ np.int64(z * P3))
    return {int(v) for v in out}


def write_backend(stem, columns, loc_attrib, time_attrib, lx, ly, lz, flush_every=5000):
    """columns: attrib id -> (type, array); type 0 = location (float x,y).
    Records are buffered per partition and every buffer is flushed when
    flush_every records are held, so partitions get several chunks."""
    ids = sorted(columns)
    ntypes = max(ids) + 1
    types = [1] * ntypes
    for a in ids:
        types[a] = columns[a][0]
    with open(stem + "_config", "wb") as f:
        f.write(struct.pack(">ddIiiiB", lx, ly, lz, P1, P2, P3, ntypes))
        f.write(bytes(types))
    xy = np.asarray(columns[loc_attrib][1], np.float32).reshape(-1, 2)
    t = np.asarray(columns[time_attrib][1], np.uint32)
    pid = partition_ids(xy[:, 0], xy[:, 1], t, lx, ly, lz)
    n = len(pid)
    # chunk plan shared by all attributes: (partition, [rows]) in write order
    chunks = []
    buf = {}
    held = 0
    for i in range(n):
        buf.setdefault(int(pid[i]), []).append(i)
        held += 1
        if held >= flush_every:
            for k in list(buf):
                if buf[k]:
                    chunks.append((k, buf[k]))
            buf = {k: [] for k in buf}
            held = 0
    for k in buf:
        if buf[k]:
            chunks.append((k, buf[k]))
    for a in ids:
        typ, arr = columns[a]
        arr = np.ascontiguousarray(arr)
        esz = 8 if typ == 0 else 4
        rows = arr.reshape(n, -1) if typ == 0 else arr
        mapping = {}
        off = 0
        with open("%s%d_payload.dat" % (stem, a), "wb") as f:
            for k, r in chunks:
                data = np.ascontiguousarray(rows[np.asarray(r)]).tobytes()
                assert len(data) == esz * len(r)
                f.write(data)
                mapping.setdefault(k, []).append((off, len(data)))
                off += len(data)
        with open("%s%d_mapping" % (stem, a), "wb") as f:
            f.write(struct.pack(">I", len(mapping)))
            for k, lst in mapping.items():
                f.write(struct.pack(">qI", k, len(lst)))
                for o, s in lst:
                    f.write(struct.pack(">QQ", o, s))
    return chunks


def selected_rows(chunks, parts):
    """Rows the reader returns for a set of partitions: chunks in file order."""
    out = []
    for k, r in chunks:
        if k in parts:
            out.extend(r)
    return np.asarray(out, np.int64)


def write_polygons(path, polys, rings=None):
    """polys: list of (n, 2) arrays; rings[i] splits polygon i into parts."""
    with open(path, "w") as f:
        f.write("%d\n" % len(polys))
        for i, p in enumerate(polys):
            parts = [p] if rings is None or rings[i] is None else np.split(p, rings[i])
            f.write("%d\n" % len(parts))
            for part in parts:
                f.write("%d\n" % len(part))
                for x, y in part:
                    f.write("%.17g %.17g\n" % (x, y))


def geo2world(lat, lon):
    """Utils.h:9-18 at zoom 22."""
    s = 2.0 ** 22
    if lat == 90.0:
        y = 256.0
    elif lat == -90.0:
        y = 0.0
    else:
        y = (np.pi - np.arctanh(np.sin(lat * np.pi / 180))) / np.pi * 128
    return (lon + 180) / 360.0 * 256 * s, y * s


def transform_point(lat, lon):
    """UsefulFuncs.cpp:578-597: world coordinates relative to the US-box centre."""
    minlat, minlon, maxlat, maxlon = 24.396308, -124.848974, 49.384358, -66.885444
    if lat < minlat or lat > maxlat or lon < minlon or lon > maxlon:
        return None
    cx, cy = geo2world((minlat + maxlat) / 2, (minlon + maxlon) / 2)
    x, y = geo2world(lat, lon)
    return x - cx, y - cy
