/* The one translation unit oracle/ref_build.py compiles to build the reference's own CUDA library
 * (pkp24/Vship src/VshipLib.cpp, staged unedited into oracle/_ref/src). Test and benchmark
 * infrastructure only: the product library never links or loads the result.
 *
 * Two additions around the reference's text, both of this project's own writing:
 *
 * 1. The reference's v2 entry points name the input types unqualified (src/VshipLib.cpp:215, :245,
 *    :323, :359: run<FLOAT>, run<UINT16>) while the enum is scoped
 *    (src/util/preprocessor.hpp:94: enum class InputMemType), so the file does not compile as
 *    shipped. Two global constants with those names, declared before the file is included, make
 *    the unqualified arguments resolve to the enum values the v1 entry points pass explicitly.
 *
 * 2. The reference's C ABI returns Butteraugli norms in a struct of ints
 *    (src/VshipAPI.h:113-117; src/VshipLib.cpp:306-308 assigns the floats to them, truncating),
 *    which is no use for a parity check at 1e-4 relative. VshipRef_ComputeButteraugli does what
 *    Vship_ComputeButteraugliUint16v2 / Floatv2 do (src/VshipLib.cpp:316-368) -- take the
 *    handler's computing implementation out of the reference's handler table and run it -- and
 *    returns the three float norms of its std::tuple result instead of the int struct. */
#include "util/preprocessor.hpp"

constexpr InputMemType FLOAT = InputMemType::FLOAT;
constexpr InputMemType UINT16 = InputMemType::UINT16;

#include "VshipLib.cpp"

extern "C" __attribute__((visibility("default")))
Vship_Exception VshipRef_ComputeButteraugli(Vship_ButteraugliHandler handler, float norms[3], int input_uint16,
                                            const uint8_t* dstp, int64_t dststride, const uint8_t* srcp1[3],
                                            const uint8_t* srcp2[3], int64_t stride, int64_t stride2) {
    Vship_Exception err = Vship_NoError;
    HandlerManagerButteraugli.lock.lock();
    if (handler.id < 0 || (size_t)handler.id >= HandlerManagerButteraugli.elements.size()) {
        HandlerManagerButteraugli.lock.unlock();
        return Vship_BadHandler;
    }
    butter::ButterComputingImplementation impl = HandlerManagerButteraugli.elements[handler.id];
    HandlerManagerButteraugli.lock.unlock();
    try {
        std::tuple<float, float, float> res =
            input_uint16 ? impl.run<InputMemType::UINT16>(dstp, dststride, srcp1, srcp2, stride, stride2)
                         : impl.run<InputMemType::FLOAT>(dstp, dststride, srcp1, srcp2, stride, stride2);
        norms[0] = std::get<0>(res);
        norms[1] = std::get<1>(res);
        norms[2] = std::get<2>(res);
    } catch (const VshipError& e) {
        err = (Vship_Exception)e.type;
    }
    return err;
}
