// rasterjoin.hpp -- C++ host interface over librj.so (include/rj.h).
//
// Mirrors the reference's host classes for the join path, with the same
// names, argument meaning and error behaviour, without Qt or OpenGL:
//   GLHandler    RasterJoin/join/GLHandler.hpp:20-78 (singleton dispatcher:
//                executeFunction -> int[3P], getErrorBounds -> int[4P],
//                printTimeStats; errors give an empty vector, as
//                GLHandler.cpp:190-203)
//   DataHandler  RasterJoin/db/DataHandler.hpp:14-41 (constraints,
//                aggregation, polygon query, the queried point table)
//   PolyHandler  RasterJoin/db/PolyHandler.hpp:28-58 (collection list and
//                polygon text files, lat/lon -> world transform)
//   QueryResult  RasterJoin/db/QueryResult.hpp:16-120 (binary columns)
//   HashGridIndex the backend column store reader (HashGridIndex.cpp,
//                BufferedPartitionedFile.cpp, PartitioningManager.cpp)
// Header-only; link with -lrj.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <unordered_set>
#include <utility>
#include <vector>

#include "rj.h"

namespace rasterjoin {

// ---- Common.h ------------------------------------------------------------
enum Aggregation { Count = RJ_COUNT, Avg = RJ_AVG, Sum = RJ_SUM };
enum ConstraintType { EQ = RJ_EQ, LT = RJ_LT, LTE = RJ_LTE, GT = RJ_GT, GTE = RJ_GTE };
enum AttributeType { Location = RJ_LOCATION, Uint = RJ_UINT, Int = RJ_INT, Float = RJ_FLOAT };
typedef rj_value Value;
typedef rj_constraint QueryConstraint;
static_assert(sizeof(QueryConstraint) == 16, "QueryConstraint is 16 bytes (main.cpp:376)");

// ---- lat/lon -> world (Utils.h:9-27, UsefulFuncs.cpp:578-632) ----------------
constexpr double kWorldZoom = 22.0;
constexpr double kMinLat = 24.396308, kMinLon = -124.848974, kMaxLat = 49.384358, kMaxLon = -66.885444;

inline void geo2world(double lat, double lon, double& x, double& y) {
    double yy;
    if (lat == 90.0) yy = 256;
    else if (lat == -90.0) yy = 0;
    else yy = (M_PI - std::atanh(std::sin(lat * M_PI / 180))) / M_PI * 128;
    const double s = std::exp2(kWorldZoom);
    x = (lon + 180) / 360.0 * 256 * s;
    y = yy * s;
}

// world coordinates relative to the centre of the continental-US box; false
// outside the box (the polygon is then dropped)
inline bool transformPoint(double lat, double lon, double& x, double& y) {
    if (lat < kMinLat || lat > kMaxLat) return false;
    if (lon < kMinLon || lon > kMaxLon) return false;
    double cx, cy, px, py;
    geo2world((kMinLat + kMaxLat) / 2, (kMinLon + kMaxLon) / 2, cx, cy);
    geo2world(lat, lon, px, py);
    x = px - cx;
    y = py - cy;
    return true;
}

// metres per world unit at the centre latitude
inline double getGroundResolution() {
    const double lat = (kMinLat + kMaxLat) / 2;
    return std::cos(lat * M_PI / 180) * 6378137 * 2 * M_PI / std::exp2(8 + kWorldZoom);
}

// ---- polygons --------------------------------------------------------------
struct Bound {
    double minx = 0, miny = 0, maxx = 0, maxy = 0;
};

struct PointD {
    double x, y;
};
typedef std::vector<PointD> TPolygon;

class PolyHandler {
public:
    // "name,file" per line; file relative to the list's directory
    // (PolyHandler::initFromFile, PolyHandler.cpp:20-40).  `geo` = false
    // reads world coordinates as they are (no lat/lon transform).
    bool initFromFile(const std::string& polyIndex, bool geo = true) {
        std::ifstream fi(polyIndex);
        if (!fi) {
            std::cerr << "Could not open file " << polyIndex << "\n";
            return false;
        }
        std::string dir = ".";
        const size_t slash = polyIndex.find_last_of('/');
        if (slash != std::string::npos) dir = polyIndex.substr(0, slash);
        std::string line;
        bool ok = true;
        while (std::getline(fi, line)) {
            if (line.find_first_not_of(" \t\r\n") == std::string::npos) continue;
            const size_t c = line.find(',');
            if (c == std::string::npos) continue;
            std::string name = line.substr(0, c), file = line.substr(c + 1);
            while (!file.empty() && (file.back() == '\r' || file.back() == ' ')) file.pop_back();
            ok = addPolygonCollection(name, dir + "/" + file, geo) && ok;
            currentCollection = name;
        }
        return ok;
    }

    // readPolygons (PolyHandler.cpp:133-188): "tot" then per polygon "np"
    // rings, each "n" followed by n "x y" pairs (lat lon when geo); rings of
    // a polygon are appended into one vertex list, repeated consecutive
    // vertices dropped, a closing vertex equal to the first removed; a
    // polygon with a vertex outside the transform's box is skipped.  Bounds
    // are accumulated in float (BoundF, Common.h:88-104).
    static bool readPolygons(const std::string& polyFile, std::vector<TPolygon>& polys, Bound& b, bool geo = true) {
        std::ifstream fi(polyFile);
        if (!fi) {
            std::cerr << "Could not open file " << polyFile << "\n";
            return false;
        }
        long tot = 0;
        fi >> tot;
        for (long i = 0; i < tot && fi; ++i) {
            long np = 0;
            fi >> np;
            TPolygon poly;
            PointD prev{0, 0};
            for (long j = 0; j < np; ++j) {
                long n = 0;
                fi >> n;
                for (long k = 0; k < n; ++k) {
                    double x, y;
                    fi >> x >> y;
                    PointD pt{x, y};
                    if (k == 0 || prev.x != pt.x || prev.y != pt.y) poly.push_back(pt);
                    prev = pt;
                }
            }
            if (poly.size() > 1 && poly.front().x == poly.back().x && poly.front().y == poly.back().y) poly.pop_back();
            TPolygon tp;
            bool keep = true;
            for (const PointD& p : poly) {
                double x = p.x, y = p.y;
                if (geo && !transformPoint(p.x, p.y, x, y)) {
                    keep = false;
                    break;
                }
                tp.push_back({x, y});
            }
            if (keep) polys.push_back(tp);
        }
        float minx = std::numeric_limits<float>::max(), miny = minx;
        float maxx = -std::numeric_limits<float>::max(), maxy = maxx;
        for (const TPolygon& p : polys)
            for (const PointD& v : p) {
                minx = std::min(minx, (float)v.x);
                maxx = std::max(maxx, (float)v.x);
                miny = std::min(miny, (float)v.y);
                maxy = std::max(maxy, (float)v.y);
            }
        b.minx = minx;
        b.miny = miny;
        b.maxx = maxx;
        b.maxy = maxy;
        return true;
    }

    bool addPolygonCollection(const std::string& name, const std::string& polyFile, bool geo = true) {
        std::vector<TPolygon> polys;
        Bound b;
        if (!readPolygons(polyFile, polys, b, geo)) return false;
        return addPolygonCollection(name, polys, b);
    }

    // flattening of PolyHandler::addPolygonCollection (PolyHandler.cpp:49-80)
    bool addPolygonCollection(const std::string& name, const std::vector<TPolygon>& polysIn, const Bound& b) {
        if (polys.count(name)) {
            std::cerr << "Collection with name " << name << " already exists!\n";
            return false;
        }
        std::vector<float> verts;
        std::vector<int> pindex;
        for (const TPolygon& p : polysIn) {
            pindex.push_back((int)(verts.size() / 2));
            for (const PointD& v : p) {
                verts.push_back((float)v.x);
                verts.push_back((float)v.y);
            }
        }
        pindex.push_back((int)(verts.size() / 2));
        polys[name] = std::move(verts);
        pindexes[name] = std::move(pindex);
        dbBounds[name] = b;
        return true;
    }

    Bound getBounds() { return dbBounds[currentCollection]; }
    int getNoPolys() { return (int)pindexes[currentCollection].size() - 1; }

    std::map<std::string, std::vector<float>> polys;
    std::map<std::string, std::vector<int>> pindexes;
    std::map<std::string, Bound> dbBounds;
    std::string currentCollection;
};

// ---- point table -------------------------------------------------------------
class QueryResult {
public:
    void addAttributeResult(size_t attrib, std::unique_ptr<std::vector<char>> result) {
        binResult[attrib] = std::move(result);
    }
    void addAttributeMetadata(size_t attrib, size_t type) { meta[attrib] = type; }
    void setLocationAttribute(size_t a) { loc = a; }
    std::vector<char>* getAttribute(size_t attrib) {
        auto it = binResult.find(attrib);
        return it == binResult.end() ? nullptr : it->second.get();
    }
    size_t getAttributeType(size_t attrib) { return meta[attrib]; }
    size_t getAttributeSize(size_t attrib) { return meta[attrib] == Location ? 8 : 4; }
    size_t getLocationAttributeId() { return loc; }
    size_t getNumAttributes() { return binResult.size(); }
    uint64_t rows() {
        auto* l = getAttribute(loc);
        return l ? l->size() / 8 : 0;
    }
    std::map<size_t, std::unique_ptr<std::vector<char>>> binResult;
    std::map<size_t, size_t> meta;
    size_t loc = 0;
};

// ---- backend column store (read side) -------------------------------------
// The reference's disk index: <stem>_config (QDataStream: lx ly as doubles,
// lz uint32, p1 p2 p3 int32, attribute count and types as quint8;
// HashGridIndex.cpp:12-33), and per attribute a <stem><id>_payload.dat of raw
// little-endian values with a <stem><id>_mapping (QDataStream of
// QHash<qint64, QVector<QPair<quint64,quint64>>>: partition -> (byte offset,
// byte size) chunks; BufferedPartitionedFile.cpp:10-51,165-200).
// QDataStream writes big-endian, containers as a quint32 count then items.
class BigEndianReader {
public:
    explicit BigEndianReader(const std::string& path) : f(path, std::ios::binary) {}
    bool ok() const { return (bool)f; }
    bool u8(uint8_t& v) { return raw(&v, 1); }
    bool u32(uint32_t& v) {
        unsigned char b[4];
        if (!raw(b, 4)) return false;
        v = (uint32_t)b[0] << 24 | (uint32_t)b[1] << 16 | (uint32_t)b[2] << 8 | b[3];
        return true;
    }
    bool u64(uint64_t& v) {
        uint32_t hi, lo;
        if (!u32(hi) || !u32(lo)) return false;
        v = (uint64_t)hi << 32 | lo;
        return true;
    }
    bool f64(double& v) {
        uint64_t u;
        if (!u64(u)) return false;
        std::memcpy(&v, &u, 8);
        return true;
    }

private:
    bool raw(void* p, size_t n) { return (bool)f.read((char*)p, (std::streamsize)n); }
    std::ifstream f;
};

class HashGridIndex {
public:
    bool open(const std::string& stem) {
        this->stem = stem;
        BigEndianReader in(stem + "_config");
        if (!in.ok()) {
            std::cerr << "Cannot open Config File\n";
            return false;
        }
        double dx, dy;
        uint32_t z, a, b, c;
        uint8_t n = 0;
        if (!in.f64(dx) || !in.f64(dy) || !in.u32(z) || !in.u32(a) || !in.u32(b) || !in.u32(c) || !in.u8(n)) return false;
        lx = (float)dx;
        ly = (float)dy;
        lz = z;
        p1 = (int32_t)a;
        p2 = (int32_t)b;
        p3 = (int32_t)c;
        types.resize(n);
        for (uint8_t i = 0; i < n; ++i)
            if (!in.u8(types[i])) return false;
        return true;
    }

    // HashGridIndex::getIntersectingPartitions (HashGridIndex.cpp:117-141):
    // float division, truncation to qint64, hashed cell ids
    void partitions(const float lo[3], const float hi[3], std::unordered_set<int64_t>& out) const {
        const int64_t x0 = (int64_t)(lo[0] / lx), y0 = (int64_t)(lo[1] / ly), z0 = (int64_t)(lo[2] / (float)lz);
        const int64_t x1 = (int64_t)(hi[0] / lx), y1 = (int64_t)(hi[1] / ly), z1 = (int64_t)(hi[2] / (float)lz);
        for (int64_t x = x0; x <= x1; ++x)
            for (int64_t y = y0; y <= y1; ++y)
                for (int64_t z = z0; z <= z1; ++z) out.insert((x * p1) ^ (y * p2) ^ (z * p3));
    }

    // BufferedPartitionedFile::getPartitions (BufferedPartitionedFile.cpp:86-133):
    // the chunks of the selected partitions in (offset, size) order
    bool readAttribute(size_t attrib, const std::unordered_set<int64_t>& parts, std::vector<char>& out) const {
        const std::string base = stem + std::to_string(attrib);
        BigEndianReader m(base + "_mapping");
        if (!m.ok()) return false;
        uint32_t n = 0;
        if (!m.u32(n)) return false;
        std::set<std::pair<uint64_t, uint64_t>> chunks;
        for (uint32_t i = 0; i < n; ++i) {
            uint64_t key;
            uint32_t cnt;
            if (!m.u64(key) || !m.u32(cnt)) return false;
            const bool want = parts.count((int64_t)key) != 0;
            for (uint32_t j = 0; j < cnt; ++j) {
                uint64_t off, sz;
                if (!m.u64(off) || !m.u64(sz)) return false;
                if (want) chunks.insert({off, sz});
            }
        }
        std::ifstream pf(base + "_payload.dat", std::ios::binary);
        if (!pf) return false;
        out.clear();
        for (const auto& c : chunks) {
            const size_t at = out.size();
            out.resize(at + c.second);
            pf.seekg((std::streamoff)c.first);
            if (!pf.read(out.data() + at, (std::streamsize)c.second)) return false;
        }
        return true;
    }

    std::string stem;
    float lx = 1, ly = 1;
    uint32_t lz = 1;
    int32_t p1 = 73856093, p2 = 19349663, p3 = 83492791;
    std::vector<uint8_t> types;
};

// ---- DataHandler -------------------------------------------------------------
class DataHandler {
public:
    // DataHandler::initData (DataHandler.cpp:24-62): polygons from the
    // collection list, point columns from the backend index
    bool initData(const std::string& polyIndex, const std::string& indexFileStem, const std::set<size_t>& attIds,
                  size_t locAtt, bool geo = true) {
        if (!polyHandler.initFromFile(polyIndex, geo)) return false;
        if (!index.open(indexFileStem)) return false;
        for (size_t i = 0; i < index.types.size(); ++i) queryResult.addAttributeMetadata(i, index.types[i]);
        queryResult.setLocationAttribute(locAtt);
        attributes.assign(1, locAtt);
        attributes.insert(attributes.end(), attIds.begin(), attIds.end());
        setAggregation();
        return true;
    }
    // DataHandler::executeQuery: the partitions of the region (x, y, time)
    bool executeQuery(const float region_low[3], const float region_high[3]) {
        std::unordered_set<int64_t> parts;
        index.partitions(region_low, region_high, parts);
        for (size_t a : attributes) {
            std::unique_ptr<std::vector<char>> col(new std::vector<char>());
            if (!index.readAttribute(a, parts, *col)) return false;
            queryResult.addAttributeResult(a, std::move(col));
        }
        ++version;
        return true;
    }
    // a point table supplied directly (no backend)
    void addAttribute(size_t attrib, AttributeType type, const void* data, uint64_t rows) {
        const size_t esz = type == Location ? 8 : 4;
        std::unique_ptr<std::vector<char>> col(new std::vector<char>((const char*)data, (const char*)data + esz * rows));
        queryResult.addAttributeMetadata(attrib, type);
        queryResult.addAttributeResult(attrib, std::move(col));
        if (type == Location) queryResult.setLocationAttribute(attrib);
        ++version;
    }
    void setQueryConstraints(std::vector<QueryConstraint> c) { constraints = std::move(c); }
    void setAggregation(Aggregation type = Count, int attribId = -1) {
        aggr = type;
        aggrAttrib = attribId;
    }
    void setPolygonQuery(const std::string& collectionName) { polyHandler.currentCollection = collectionName; }
    // exact inclusive time range on a uint column (DataHandler.cpp:107-109);
    // attrib < 0 turns it off
    void setTimeRange(int attrib, uint32_t start, uint32_t end) {
        timeAttrib = attrib;
        tStart = start;
        tEnd = end;
    }
    QueryResult* getCoarseQueryResult() { return &queryResult; }
    PolyHandler* getPolyHandler() { return &polyHandler; }
    std::vector<QueryConstraint> getQueryConstraints() { return constraints; }
    void getAggregation(Aggregation& type, int& attribId) {
        type = aggr;
        attribId = aggrAttrib;
    }

    QueryResult queryResult;
    PolyHandler polyHandler;
    HashGridIndex index;
    std::vector<size_t> attributes;
    std::vector<QueryConstraint> constraints;
    Aggregation aggr = Count;
    int aggrAttrib = -1;
    int timeAttrib = -1;
    uint32_t tStart = 0, tEnd = 0;
    uint64_t version = 0;
};

// ---- GLHandler ---------------------------------------------------------------
class GLHandler {
public:
    enum FunctionType { RasterJoinFn = 0, IndexJoinFn, HybridJoinFn, RasterJoinBoundFn, FunctionCount };

    // singleton as GLHandler::getInstance (GLHandler.cpp:64-69); NULL when no
    // CUDA device can be used
    static GLHandler* getInstance(int64_t gpuMemMB = 2048LL, bool inMemory = false) {
        static std::unique_ptr<GLHandler> inst;
        if (!inst) {
            std::unique_ptr<GLHandler> h(new GLHandler());
            rj_config cfg{0, gpuMemMB, nullptr};
            if (rj_create(&cfg, &h->ctx) != RJ_OK) return nullptr;
            h->inmem = inMemory ? 1 : 0;
            inst = std::move(h);
        }
        return inst.get();
    }
    ~GLHandler() {
        if (ctx) rj_destroy(ctx);
    }

    void setDataHandler(DataHandler* dh) { dataHandler = dh; }
    void setAccuracyDistance(double size) {
        accuracy = (int)size;
        accuracyDistance = size;
    }
    void setPolyIndexResolution(int resx, int resy) {
        presx = resx;   // only x is used (GLFunction.cpp:76)
        presy = resy;
    }
    // explicit pixel side in world units (overrides the accuracy distance)
    void setCellSize(double cell) { cellSize = cell; }

    // GLHandler::executeFunction (GLHandler.cpp:188-204): [count | sum/100 |
    // decimal*10] per polygon; an empty vector on error
    std::vector<int> executeFunction(FunctionType fn) {
        bounds.clear();
        if (!run(fn)) return std::vector<int>();
        return compat3;
    }
    // GLHandler::getErrorBounds (GLHandler.cpp:206-212): [fn | fp | fn1 | fp1]
    std::vector<int> getErrorBounds(FunctionType fn) {
        return fn == RasterJoinBoundFn ? bounds : std::vector<int>();
    }
    // GLHandler::printTimeStats (GLHandler.cpp:214-248)
    std::string printTimeStats(FunctionType) {
        char buf[512];
        if (rj_format_time_stats(ctx, buf, sizeof buf) != RJ_OK) return std::string();
        return buf;
    }
    const char* lastError() const { return rj_last_error(ctx); }

    // exact per-polygon results of the last call
    std::vector<uint64_t> counts;
    std::vector<double> sums;

    rj_ctx* ctx = nullptr;
    DataHandler* dataHandler = nullptr;
    int presx = 256, presy = 256;
    int inmem = 0;
    int accuracy = 100;
    double accuracyDistance = 100.0;
    double cellSize = 0.0;
    double groundResolution = 1.0;     // metres per world unit (getGroundResolution() for geo data)
    uint32_t flags = 0;                // RJ_FLAG_*

private:
    GLHandler() = default;

    bool upload() {
        DataHandler* dh = dataHandler;
        QueryResult& qr = dh->queryResult;
        if (dh->version != loadedVersion) {
            std::vector<rj_column> cols;
            uint64_t n = qr.rows();
            for (auto& kv : qr.binResult) {
                const size_t type = qr.getAttributeType(kv.first);
                cols.push_back({(int32_t)kv.first, (int32_t)type, kv.second->data()});
            }
            if (rj_load_points(ctx, cols.data(), (int32_t)cols.size(), n, (int32_t)qr.getLocationAttributeId()) != RJ_OK)
                return false;
            loadedVersion = dh->version;
        }
        PolyHandler& ph = dh->polyHandler;
        if (ph.currentCollection != loadedCollection) {
            const std::vector<float>& v = ph.polys[ph.currentCollection];
            const std::vector<int>& p = ph.pindexes[ph.currentCollection];
            const Bound b = ph.getBounds();
            const double bb[4] = {b.minx, b.miny, b.maxx, b.maxy};
            if (p.size() < 2 || rj_set_polygons(ctx, v.data(), p.data(), (int32_t)p.size() - 1, bb) != RJ_OK)
                return false;
            loadedCollection = ph.currentCollection;
        }
        return true;
    }

    bool run(FunctionType fn) {
        if (!dataHandler) {
            std::cerr << "DataHandler not set\n";
            return false;
        }
        if (!upload()) {
            std::cerr << rj_last_error(ctx) << "\n";
            return false;
        }
        rj_query q;
        rj_query_init(&q);
        q.function_type = fn;
        Aggregation ag;
        int aa;
        dataHandler->getAggregation(ag, aa);
        q.aggregation = ag;
        q.aggr_attrib = aa;
        const std::vector<QueryConstraint>& cs = dataHandler->constraints;
        q.n_constraints = (int32_t)cs.size();
        for (size_t i = 0; i < cs.size() && i < RJ_MAX_CONSTRAINTS; ++i) q.constraints[i] = cs[i];
        q.accuracy_m = accuracyDistance;
        q.cell_size = cellSize;
        q.ground_resolution = groundResolution;
        q.grid_res = presx;
        q.time_attrib = dataHandler->timeAttrib;
        q.t_start = dataHandler->tStart;
        q.t_end = dataHandler->tEnd;
        q.flags = flags;
        const int P = dataHandler->polyHandler.getNoPolys();
        counts.assign(P, 0);
        sums.assign(P, 0.0);
        compat3.assign(3 * (size_t)P, 0);
        bounds.assign(4 * (size_t)P, 0);
        rj_result r{P, counts.data(), sums.data(), compat3.data(), fn == RasterJoinBoundFn ? bounds.data() : nullptr};
        const int rc = rj_execute(ctx, &q, &r);
        if (rc != RJ_OK) {
            std::cerr << "join failed (" << rc << "): " << rj_last_error(ctx) << "\n";
            compat3.clear();
            bounds.clear();
            return false;
        }
        if (fn != RasterJoinBoundFn) bounds.clear();
        return true;
    }

    std::vector<int> compat3, bounds;
    uint64_t loadedVersion = ~0ULL;
    std::string loadedCollection;
};

}  // namespace rasterjoin
