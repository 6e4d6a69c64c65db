// ose_io.h - SU / SEG-Y trace writers (ose_io.cpp).
#pragma once

namespace ose {

// Geometry of one shot gather; distances in metres.
struct TraceGeometry {
    int ng, nt, nx;        // traces, samples per trace, receivers per row (ig = iy*nx + ix)
    int shot;              // shot index (fldr = shot + 1)
    double dx, dy;         // receiver spacing
    double sx, sy, sz;     // source position
    double gz;             // receiver depth
    int dt_us;             // sample interval in microseconds
    const int* rxyz;       // receiver list: (x, y, z) interior cells per trace, or
                           // null for the receiver plane (ig = iy * nx + ix, depth gz)
    double dz;
};

// Writes ng traces of nt samples from gather_ig_it ([ig][it]); segy = false
// gives SU (native byte order, no file header).  0 on success, -1 on I/O
// error, -2 when nt or the sample interval do not fit the 16-bit header fields.
int write_gather_traces(const char* path, const float* gather_ig_it, const TraceGeometry& g, bool segy);

}  // namespace ose
