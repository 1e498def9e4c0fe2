// tri_wrap.cpp -- C entry point around the reference's polygon triangulation
// (clip2tri: clipper union + poly2tri constrained Delaunay), called the way
// PolyHandler::getTriangulation does (RasterJoin/db/PolyHandler.cpp:82-115):
// one polygon per call, no bounding polygon.  TEST INFRASTRUCTURE ONLY: it is
// linked with the reference's own sources into oracle/_ref/libreftri.so and
// used by the fill-rule cross-check in tests/; nothing in the library uses it.
#include <vector>

#include "clip2tri/clip2tri.h"

extern "C" int ref_triangulate(const double* xy, int n, double* out, int cap_triangles) {
    std::vector<std::vector<c2t::Point>> in(1);
    for (int i = 0; i < n; ++i) in[0].push_back(c2t::Point(xy[2 * i], xy[2 * i + 1]));
    std::vector<c2t::Point> tris, bounding;
    c2t::clip2tri c;
    c.triangulate(in, tris, bounding);
    const int nt = (int)tris.size() / 3;
    if (nt > cap_triangles) return -nt;
    for (size_t k = 0; k < tris.size(); ++k) {
        out[2 * k] = tris[k].x;
        out[2 * k + 1] = tris[k].y;
    }
    return nt;
}
