// Drives one ping through the C++ mirror of the reference's receiver API
// (include/rtacx/simulation.hpp) the way code written for rtac_simulation
// would: SensorInfo + Waveform_Sine + BeamDirectivity -> SensorInstance,
// set_sample_count, fill samples(), compute_output(), read output().
//
// usage: sensor_instance_demo <params.txt> <samples.bin> <out.bin> [sink]
// With [sink], a 2D ping is computed twice and appended twice to a FileSink.
// params.txt holds "key value" lines (dims, range_min, range_max,
// range_count, celerity, frequency, duration, fixed, oversampling,
// beam_span) and "key n v_0 .. v_n-1" lines (beam, bearings).
// samples.bin: float32 AoS records (12 B 1D, 16 B 2D); out.bin: complex64.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include <rtacx/simulation.hpp>

using namespace rtacx::simulation;

int main(int argc, char** argv)
{
    if(argc != 4 && argc != 5) { std::cerr << "usage: " << argv[0] << " params.txt samples.bin out.bin [sink]\n"; return 2; }
    std::map<std::string, double> scalars;
    std::map<std::string, std::vector<float>> arrays;
    std::ifstream pf(argv[1]);
    std::string line;
    while(std::getline(pf, line)) {
        std::istringstream in(line);
        std::string key; in >> key;
        if(key == "beam" || key == "bearings") {
            size_t n; in >> n;
            std::vector<float> v(n);
            for(auto& x : v) in >> x;
            arrays[key] = v;
        }
        else if(!key.empty()) { double v; in >> v; scalars[key] = v; }
    }
    std::ifstream sf(argv[2], std::ios::binary);
    std::vector<char> raw((std::istreambuf_iterator<char>(sf)), std::istreambuf_iterator<char>());
    try {
        const Linspace ranges((float)scalars["range_min"], (float)scalars["range_max"], (unsigned)scalars["range_count"]);
        auto waveform = Waveform_Sine::Create((float)scalars["frequency"], (float)scalars["duration"],
                                              scalars["fixed"] != 0.0, (unsigned)scalars["oversampling"]);
        std::vector<Complex> out;
        if((int)scalars["dims"] == 2) {
            auto beam = BeamDirectivity::Create((float)scalars["beam_span"], arrays["beam"]);
            auto info = SensorInfo2D::Create(arrays["bearings"], ranges, waveform, beam);
            const size_t n = raw.size() / sizeof(SimSample2D);
            if(argc == 5) {
                // The reference factory's spelling: SensorInstance2D_2<Complex<float>>, read through get_ping().
                auto sensor = SensorInstance2D_2<Complex>::Create(SensorInfo::ConstPtr(info), (float)scalars["celerity"]);
                sensor->set_sample_count((unsigned)n);
                sensor->samples().copy_from_host(reinterpret_cast<const SimSample2D*>(raw.data()), n);
                sensor->compute_output();
                const Ping2D ping = sensor->get_ping();
                if(ping.width() != sensor->width() || ping.height() != sensor->height() || !sensor->is_complex())
                    throw std::runtime_error("get_ping geometry");
                out = ping.to_host();
                auto sink = FileSink::Create(argv[4], true);
                sink->set_output(sensor);
                sensor->compute_output();
                sink->set_output(sensor);
            }
            else {
                auto sensor = SensorInstance2D_Complex::Create(SensorInfo2D::ConstPtr(info), (float)scalars["celerity"]);
                if(scalars["texture_psf"] != 0.0) sensor->set_texture_psf(true);
                sensor->set_sample_count((unsigned)n);
                sensor->samples().copy_from_host(reinterpret_cast<const SimSample2D*>(raw.data()), n);
                sensor->compute_output();
                out = sensor->output().to_host();
            }
        }
        else {
            auto info = SensorInfo::Create(ranges, waveform);
            auto sensor = SensorInstance1D_Complex::Create(info, (float)scalars["celerity"]);
            const size_t n = raw.size() / sizeof(SimSample1D);
            sensor->set_sample_count((unsigned)n);
            sensor->samples().copy_from_host(reinterpret_cast<const SimSample1D*>(raw.data()), n);
            sensor->compute_output();
            out = sensor->output().to_host();
        }
        std::ofstream of(argv[3], std::ios::binary);
        of.write(reinterpret_cast<const char*>(out.data()), out.size() * sizeof(Complex));
    }
    catch(const std::exception& e) {
        std::cerr << "error: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
