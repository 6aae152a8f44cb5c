// Compile check of the librtacx binding against the reference's own headers.
//
// The binding statements (sensor_instance2d_rtacx.inc) are compiled inside a
// class derived from the reference's SensorInstance2D_Complex
// (include/rtac_simulation/SensorInstance2D.h:146-196), so every member they
// touch (ranges_, waveform_, info_, soundCelerity_, receivedSamples_) has the
// reference's declared type. The non-vendored rtac_base headers are the
// stand-ins of oracle/ref_stubs_binding and oracle/ref_stubs. The layout of
// the reference's sample record is checked against the 16-byte record the
// library reads. Built by tests/test_binding.py with g++ -c, then linked
// into a shared object against librtacx.so (the reference's own symbols stay
// undefined: this file is compiled, not run).
#include <stdexcept>
#include <vector>
#include <cstddef>

#include <rtac_simulation/SensorInstance.h>
#include <rtacx.h>

namespace rtac { namespace simulation {

class RtacxBoundSensorInstance2D : public SensorInstance2D_Complex
{
    public:
#include "sensor_instance2d_rtacx.inc"
};

static_assert(sizeof(SimSample2D) == 16, "the library reads 16-byte 2D records");
static_assert(offsetof(SimSample2D, value_) == 0, "record: complex value first");
static_assert(offsetof(SimSample2D, travel_) == 8, "record: travel at byte 8");
static_assert(offsetof(SimSample2D, bearing_) == 12, "record: bearing at byte 12");
static_assert(sizeof(SimSample1D) == 12, "the library reads 12-byte 1D records");
static_assert(offsetof(SimSample1D, travel_) == 8, "1D record: travel at byte 8");

}}

// The ping type of SensorInstance2D_Complex::get_ping().
template void rtac::simulation::RtacxBoundSensorInstance2D::fill_ping_rtacx<rtac::Complex<float>>(
    rtac::cuda::CudaPing2D<rtac::Complex<float>>&, bool);

extern "C" void rtacx_binding_compile_check(rtac::simulation::RtacxBoundSensorInstance2D* s,
                                            rtac::cuda::CudaPing2D<rtac::Complex<float>>* ping)
{
    s->generate_psf_data_rtacx();
    s->fill_ping_rtacx(*ping);
    s->release_rtacx();
}
