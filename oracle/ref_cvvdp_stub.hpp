/* Stands in for the reference's src/cvvdp/vapoursynth.hpp when oracle/ref_build.py compiles the
 * reference's own CUDA library. Test and benchmark infrastructure only.
 *
 * CVVDP is a third metric, outside the scored path, and needs rapidjson, which the reference does
 * not vendor (src/cvvdp/config.hpp:15). src/VshipLib.cpp:5 includes this header and :62 registers
 * cvvdp::cvvdpCreate as a VapourSynth filter; this stand-in provides that one symbol, which
 * reports that the filter is absent. Nothing on the SSIMULACRA2 / Butteraugli path uses it. */
#pragma once
#include "VapourSynth4.h"

namespace cvvdp {
static void VS_CC cvvdpCreate(const VSMap*, VSMap* out, void*, VSCore*, const VSAPI* vsapi) {
    vsapi->mapSetError(out, "CVVDP is not part of this build");
}
}  // namespace cvvdp
