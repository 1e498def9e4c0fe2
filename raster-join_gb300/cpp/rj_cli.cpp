// rj_cli -- command-line driver with the reference's options and outputs
// (RasterJoin/main.cpp:61-345): the same flags, the same result files
// (raster_<end>_<accuracy>.csv, err_bound_<end>_<accuracy>.csv) and the
// same tab-separated timing line (GLHandler::printTimeStats), so the
// reference's experiment scripts and plot parsers read its output unchanged.
//
//   rj_cli --joinType raster|hybrid|index|errorbounds --backendIndexName STEM
//          --polygonList LIST --polygonDataset NAME --locAttrib ID
//          --startTime T0 --endTime T1 [--accuracy M] [--indexRes R]
//          [--nAttrib K] [--avg ID] [--nIter N] [--opAggregation DIR]
//          [--outputTime FILE] [--gpuMem MB] [--inmem] [--inputSize N]
// Options that do not exist in the reference:
//          --world          polygon files hold world coordinates (no lat/lon
//                           transform; ground resolution 1)
//          --cellSize C     pixel side in world units instead of --accuracy
//          --exactTime ID   also keep only points with ID in [T0, T1]
//                           (the backend selects whole time partitions)
//          --dumpOnly       load polygons and points, print a summary, no join
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <string>

#include "rasterjoin.hpp"

using namespace rasterjoin;

namespace {

std::map<std::string, std::string> parse(int argc, char** argv) {
    // "--key value", or "--key" alone when the next word is another option
    // (main.cpp:383-396)
    std::map<std::string, std::string> args;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        if (a.rfind("--", 0) != 0) continue;
        std::string v = " ";
        if (i + 1 < argc) v = argv[i + 1];
        if (v.rfind("--", 0) == 0) v = " ";
        args[a] = v;
    }
    return args;
}

// setupConstraints (main.cpp:81-110): the taxi experiment's filters
std::vector<QueryConstraint> taxi_constraints(int nAttrib) {
    std::vector<QueryConstraint> c;
    auto add = [&](int attrib, ConstraintType t, Value v) {
        QueryConstraint q{};
        q.attrib_id = attrib;
        q.type = t;
        q.val = v;
        c.push_back(q);
    };
    Value v;
    if (nAttrib >= 1) { v.uval = 1; add(18, EQ, v); }      // passengers
    if (nAttrib >= 2) { v.uval = 1000; add(8, GT, v); }    // fare
    if (nAttrib >= 3) { v.fval = 10.f; add(7, LT, v); }    // miles
    if (nAttrib == 4) { v.uval = 20; add(6, GT, v); }      // duration
    return c;
}

GLHandler::FunctionType join_operator(const std::string& j, bool& ok) {
    ok = true;
    if (j == "raster") return GLHandler::RasterJoinFn;
    if (j == "hybrid") return GLHandler::HybridJoinFn;
    if (j == "index") return GLHandler::IndexJoinFn;
    if (j == "errorbounds") return GLHandler::RasterJoinBoundFn;
    ok = false;
    return GLHandler::RasterJoinFn;
}

}  // namespace

int main(int argc, char** argv) {
    auto args = parse(argc, argv);
    auto has = [&](const char* k) { return args.count(k) != 0; };
    auto str = [&](const char* k) {
        std::string s = args[k];
        while (!s.empty() && s.back() == ' ') s.pop_back();
        while (!s.empty() && s.front() == ' ') s.erase(0, 1);
        return s;
    };
    static const char* required[] = {"--joinType", "--backendIndexName", "--polygonList", "--polygonDataset",
                                     "--locAttrib", "--startTime", "--endTime"};
    bool ok = !has("--help");
    for (const char* r : required) ok = ok && has(r);
    if (!ok) {
        std::cout << "help message: see code!" << "\n";
        return 1;
    }
    const size_t nIter = has("--nIter") ? std::stoul(str("--nIter")) : 1;
    int accuracy = has("--accuracy") ? std::stoi(str("--accuracy")) : 100;
    const std::string joinType = str("--joinType");
    const int gridRes = has("--indexRes") ? std::stoi(str("--indexRes")) : 256;
    const int nAttrib = has("--nAttrib") ? std::stoi(str("--nAttrib")) : 0;
    const uint32_t start_time = (uint32_t)std::stoll(str("--startTime"));
    const uint32_t end_time = (uint32_t)std::stoll(str("--endTime"));
    const bool inMemory = has("--inmem");
    const bool opAgg = has("--opAggregation");
    const std::string aggFile = opAgg ? str("--opAggregation") : "";
    const int aggrAttrib = has("--avg") ? std::stoi(str("--avg")) : -1;
    const bool opTime = has("--outputTime");
    const std::string timeFile = opTime ? str("--outputTime") : "";
    const int64_t gpuMem = has("--gpuMem") ? std::stoll(str("--gpuMem")) : 8LL * 256LL;
    const bool world = has("--world");
    const size_t loc = std::stoul(str("--locAttrib"));
    bool jok;
    const GLHandler::FunctionType fn = join_operator(joinType, jok);
    if (!jok) {
        std::cerr << "Wrong join type " << std::endl;
        return 1;
    }

    std::set<size_t> attributes;
    std::vector<QueryConstraint> constraints;
    if (nAttrib > 0) {
        constraints = taxi_constraints(nAttrib);
        for (const QueryConstraint& c : constraints) attributes.insert((size_t)c.attrib_id);
    }
    if (aggrAttrib != -1) attributes.insert((size_t)aggrAttrib);
    if (has("--exactTime")) attributes.insert(std::stoul(str("--exactTime")));

    // setupExperiment (main.cpp:120-150)
    DataHandler dh;
    if (!dh.initData(str("--polygonList"), str("--backendIndexName"), attributes, loc, !world)) {
        std::cerr << "could not load the polygons or the backend index\n";
        return 1;
    }
    dh.setPolygonQuery(str("--polygonDataset"));
    const Bound b = dh.getPolyHandler()->getBounds();
    const float lo[3] = {(float)b.minx, (float)b.miny, (float)start_time};
    const float hi[3] = {(float)b.maxx, (float)b.maxy, (float)end_time};
    if (!dh.executeQuery(lo, hi)) {
        std::cerr << "backend query failed\n";
        return 1;
    }
    if (nAttrib > 0) dh.setQueryConstraints(constraints);
    if (aggrAttrib != -1) dh.setAggregation(Avg, aggrAttrib);
    if (has("--exactTime")) dh.setTimeRange(std::stoi(str("--exactTime")), start_time, end_time);

    if (has("--dumpOnly")) {
        QueryResult* qr = dh.getCoarseQueryResult();
        std::printf("polygons %d vertices %zu bounds %.9g %.9g %.9g %.9g rows %llu\n",
                    dh.getPolyHandler()->getNoPolys(), dh.getPolyHandler()->polys[str("--polygonDataset")].size() / 2,
                    b.minx, b.miny, b.maxx, b.maxy, (unsigned long long)qr->rows());
        for (auto& kv : qr->binResult) {
            uint64_t h = 1469598103934665603ULL;   // FNV-1a of the column bytes
            for (char c : *kv.second) h = (h ^ (unsigned char)c) * 1099511628211ULL;
            std::printf("attr %zu bytes %zu fnv %016llx\n", kv.first, kv.second->size(), (unsigned long long)h);
        }
        return 0;
    }

    GLHandler* handler = GLHandler::getInstance(gpuMem, inMemory);
    if (handler == nullptr) {
        std::cout << "Failed to obtain handler";
        return 1;
    }
    handler->setDataHandler(&dh);
    handler->setAccuracyDistance(accuracy);
    handler->setPolyIndexResolution(gridRes, gridRes);
    handler->groundResolution = world ? 1.0 : getGroundResolution();
    if (has("--cellSize")) handler->setCellSize(std::stod(str("--cellSize")));

    // runExperiment (main.cpp:168-176)
    std::vector<int> agg, bounds;
    for (size_t k = 0; k < nIter; ++k) {
        agg = handler->executeFunction(fn);
        bounds = handler->getErrorBounds(fn);
        if (agg.empty()) return 1;
    }

    // outputResults (main.cpp:227-252)
    if (opAgg) {
        if (fn != GLHandler::RasterJoinFn && fn != GLHandler::RasterJoinBoundFn) accuracy = 0;
        const int np = (int)agg.size() / 3;
        if (fn == GLHandler::RasterJoinBoundFn) {
            // outputErrorBounds (main.cpp:178-193)
            const std::string name = aggFile + "/err_bound_" + std::to_string(end_time) + "_" + std::to_string(accuracy) + ".csv";
            FILE* f = std::fopen(name.c_str(), "w");
            if (f) {
                const int nb = (int)bounds.size() / 4;
                for (int i = 0; i < nb; ++i) {
                    const int fnv = bounds[i], fp = bounds[i + nb], fn1 = bounds[i + 2 * nb], fp1 = bounds[i + 3 * nb];
                    std::fprintf(f, "%d\t%d\t%d\t%d\t%d\n", i, agg[i] - fp1, agg[i] + fn1, agg[i] - fp, agg[i] + fnv);
                }
                std::fclose(f);
            }
        } else {
            // printResults (main.cpp:195-225)
            const bool to_file = end_time > 0;
            FILE* f = stdout;
            if (to_file) {
                const std::string name = aggFile + "/raster_" + std::to_string(end_time) + "_" + std::to_string(accuracy) + ".csv";
                f = std::fopen(name.c_str(), "w");
            }
            if (f) {
                for (int i = 0; i < np; ++i) {
                    if (aggrAttrib == -1) {
                        std::fprintf(f, to_file ? "%d\t%d\n" : "%d\t%d\t\n", i, agg[i]);
                    } else {
                        const float num = float(agg[np + i]) * 100.f + agg[2 * np + i] / 10.f;
                        const float den = (float)agg[i];
                        const float avg = (agg[i] == 0) ? 0.f : num / den;
                        std::fprintf(f, "%d\t%.10g\n", i, (double)avg);
                    }
                }
                if (to_file) std::fclose(f);
            }
        }
    }
    const std::string timing = handler->printTimeStats(fn);
    if (opTime) {
        std::ofstream fo(timeFile, std::ios::app);
        if (!fo) std::cerr << "could not open file for writing: " << timeFile << "\n";
        fo << timing << "\n";
    }
    return 0;
}
