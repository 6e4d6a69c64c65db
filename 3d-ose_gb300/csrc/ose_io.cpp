// ose_io.cpp - trace output of a shot gather in the SU and SEG-Y formats.
//
// The reference links CWP/SU (Makefile:5) and names an .su model
// (ose_3d.cu:17-18, .MISSING_LARGE_BLOBS), but writes its gather as raw floats
// only (write_3dfile_from_1darray, ose_3d_lib.cu:327-343).  These writers add
// the trace headers: SU = 240-byte SEG-Y trace header + samples, native byte
// order, no file header; SEG-Y = 3200-byte text header + 400-byte binary
// header + big-endian traces of IEEE floats (format code 5).
#include "ose_io.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <vector>

namespace ose {
namespace {

template <typename T>
void put(unsigned char* h, int off, T v, bool big)
{
    unsigned char b[sizeof(T)];
    memcpy(b, &v, sizeof(T));
    if (big)
        for (size_t i = 0; i < sizeof(T); ++i) h[off + i] = b[sizeof(T) - 1 - i];
    else
        memcpy(h + off, b, sizeof(T));
}

void fill_trace_header(unsigned char* h, const TraceGeometry& g, int ig, bool big)
{
    memset(h, 0, 240);
    const int ix = g.rxyz ? g.rxyz[3 * ig] : ig % g.nx, iy = g.rxyz ? g.rxyz[3 * ig + 1] : ig / g.nx;
    const double gx = (double)ix * g.dx, gy = (double)iy * g.dy;
    const double gzr = g.rxyz ? (double)g.rxyz[3 * ig + 2] * g.dz : g.gz;
    const double ox = gx - g.sx, oy = gy - g.sy;
    const int32_t scale = -100;   // coordinates stored in centimetres (value / 100)
    put<int32_t>(h, 0, ig + 1, big);                    // tracl
    put<int32_t>(h, 4, ig + 1, big);                    // tracr
    put<int32_t>(h, 8, g.shot + 1, big);                // fldr
    put<int32_t>(h, 12, ig + 1, big);                   // tracf
    put<int32_t>(h, 16, g.shot + 1, big);               // ep
    put<int16_t>(h, 28, 1, big);                        // trid: seismic data
    put<int32_t>(h, 36, (int32_t)(100.0 * sqrt(ox * ox + oy * oy) + 0.5), big);  // offset
    put<int32_t>(h, 40, (int32_t)(-100.0 * gzr + (gzr >= 0 ? -0.5 : 0.5)), big);         // gelev
    put<int32_t>(h, 48, (int32_t)(100.0 * g.sz + 0.5), big);                               // sdepth
    put<int16_t>(h, 68, (int16_t)scale, big);           // scalel
    put<int16_t>(h, 70, (int16_t)scale, big);           // scalco
    put<int32_t>(h, 72, (int32_t)(100.0 * g.sx + 0.5), big);   // sx
    put<int32_t>(h, 76, (int32_t)(100.0 * g.sy + 0.5), big);   // sy
    put<int32_t>(h, 80, (int32_t)(100.0 * gx + 0.5), big);     // gx
    put<int32_t>(h, 84, (int32_t)(100.0 * gy + 0.5), big);     // gy
    put<int16_t>(h, 88, 1, big);                                // counit: length (m)
    put<uint16_t>(h, 114, (uint16_t)g.nt, big);                 // ns
    put<uint16_t>(h, 116, (uint16_t)(g.dt_us), big);            // dt (us)
}

}  // namespace

int write_gather_traces(const char* path, const float* gather_ig_it, const TraceGeometry& g, bool segy)
{
    if (g.nt > 65535 || g.dt_us > 65535 || g.dt_us < 1) return -2;
    FILE* f = fopen(path, "wb");
    if (!f) return -1;
    bool ok = true;
    if (segy) {
        char text[3200];
        memset(text, ' ', sizeof text);
        char line[81];
        const char* lines[] = {"C01 OSE 3D ACOUSTIC MODELING SHOT GATHER (ose3d-gb300)",
                               "C02 RECEIVER Q FIELD, ONE TRACE PER SURFACE CELL, TRACE ORDER IG = IY*NX + IX",
                               "C03 SAMPLE FORMAT IEEE FLOAT (CODE 5), BIG ENDIAN, COORDINATES IN CM",
                               "C40 END TEXTUAL HEADER"};
        for (int i = 0; i < 4; ++i) {
            const int row = i == 3 ? 39 : i;
            snprintf(line, sizeof line, "%-80s", lines[i]);
            memcpy(text + 80 * row, line, 80);
        }
        ok = ok && fwrite(text, 1, sizeof text, f) == sizeof text;
        unsigned char bin[400];
        memset(bin, 0, sizeof bin);
        put<int32_t>(bin, 0, 1, true);                          // job id
        put<int32_t>(bin, 4, 1, true);                          // line number
        put<int32_t>(bin, 8, 1, true);                          // reel number
        put<int16_t>(bin, 12, (int16_t)(g.ng > 32767 ? 0 : g.ng), true);   // traces per ensemble
        put<uint16_t>(bin, 16, (uint16_t)g.dt_us, true);        // sample interval (us)
        put<uint16_t>(bin, 20, (uint16_t)g.nt, true);           // samples per trace
        put<int16_t>(bin, 24, 5, true);                         // format: IEEE float
        put<int16_t>(bin, 28, 1, true);                         // sorting: as recorded
        put<int16_t>(bin, 54, 1, true);                         // measurement system: metres
        put<uint16_t>(bin, 300, 0x0100, true);                  // SEG-Y revision 1.0
        put<int16_t>(bin, 302, 1, true);                        // fixed trace length
        ok = ok && fwrite(bin, 1, sizeof bin, f) == sizeof bin;
    }
    std::vector<unsigned char> tr(240 + sizeof(float) * (size_t)g.nt);
    for (int ig = 0; ig < g.ng && ok; ++ig) {
        fill_trace_header(tr.data(), g, ig, segy);
        const float* s = gather_ig_it + (size_t)ig * g.nt;
        if (segy) {
            for (int t = 0; t < g.nt; ++t) put<float>(tr.data(), 240 + 4 * t, s[t], true);
        } else {
            memcpy(tr.data() + 240, s, sizeof(float) * (size_t)g.nt);
        }
        ok = fwrite(tr.data(), 1, tr.size(), f) == tr.size();
    }
    if (fclose(f) != 0) ok = false;
    return ok ? 0 : -1;
}

}  // namespace ose
