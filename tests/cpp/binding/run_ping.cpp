// Runs one 2D ping through the librtacx binding statements
// (sensor_instance2d_rtacx.inc) on a GPU. The class below stands in for the
// reference's SensorInstance2D with its member names and the accessors the
// binding uses (real_headers.cpp compiles the same statements against the
// reference's own headers where the reference tree is present). The caller
// compares the ping with the oracle.
//
//   run_ping PARAMS SAMPLES OUT [texture]
// PARAMS: text lines "range_min v", "range_max v", "range_count n",
// "celerity v", "duration v", "beam_span v", "pulse n re im ...",
// "beam n v ...", "bearings n v ..."; SAMPLES: float32 records
// {re, im, travel, bearing}; OUT: complex64 ping, range-major.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>
#include <complex>

#include <cuda_runtime.h>
#include <rtacx.h>

namespace rtac {
template <typename T> using Complex = std::complex<T>;
template <typename T> struct Bounds { T lower, upper; };
template <typename T> struct Linspace {
    T lower_, upper_; unsigned int size_;
    Bounds<T> bounds() const { return Bounds<T>{lower_, upper_}; }
    unsigned int size() const { return size_; }
};
template <typename T> using HostVector = std::vector<T>;
namespace cuda {
// Device vector: the samples and the ping live in device memory, as in the
// reference.
template <typename T> struct CudaVector {
    T* ptr = nullptr; std::size_t n = 0;
    void resize(std::size_t m) {
        if(ptr) cudaFree(ptr);
        ptr = nullptr; n = m;
        if(m && cudaMalloc(&ptr, m * sizeof(T)) != cudaSuccess) throw std::runtime_error("cudaMalloc failed");
    }
    ~CudaVector() { if(ptr) cudaFree(ptr); }
    T* data() { return ptr; }
    const T* data() const { return ptr; }
    std::size_t size() const { return n; }
};
template <typename T> struct CudaPing2D {
    Linspace<float> ranges_{}; std::size_t bearings_ = 0; CudaVector<T> data_;
    void set_bearings(const HostVector<float>& b, bool resize) { bearings_ = b.size(); if(resize) data_.resize(ranges_.size() * bearings_); }
    void set_ranges(const Linspace<float>& r, bool resize) { ranges_ = r; if(resize) data_.resize(ranges_.size() * bearings_); }
    CudaVector<T>& ping_data_container() { return data_; }
};
}
namespace simulation {
struct Waveform {
    std::vector<Complex<float>> taps; float duration_;
    unsigned int size() const { return (unsigned int)taps.size(); }
    Complex<float> operator[](unsigned int i) const { return taps[i]; }
    float duration() const { return duration_; }
};
struct BeamDirectivity {
    std::vector<float> values; float span_;
    unsigned int size() const { return (unsigned int)values.size(); }
    float operator[](unsigned int i) const { return values[i]; }
    float span() const { return span_; }
};
struct SensorInfo2D {
    HostVector<float> bearings_; std::shared_ptr<const BeamDirectivity> beam_;
    const HostVector<float>& bearings() const { return bearings_; }
    std::shared_ptr<const BeamDirectivity> beam_directivity() const { return beam_; }
};
struct SimSample2D { Complex<float> value_; float travel_; float bearing_; };

class BoundSensorInstance2D {
    public:
    Linspace<float> ranges_{};
    std::shared_ptr<Waveform> waveform_;
    std::shared_ptr<const SensorInfo2D> info_;
    float soundCelerity_ = 1500.0f;
    cuda::CudaVector<SimSample2D> receivedSamples_;
#include "sensor_instance2d_rtacx.inc"
};
}}

using namespace rtac;
using namespace rtac::simulation;

int main(int argc, char** argv)
{
    if(argc < 4) { std::cerr << "usage: run_ping PARAMS SAMPLES OUT [texture]\n"; return 2; }
    try {
        std::ifstream pf(argv[1]);
        std::map<std::string, std::vector<double>> p;
        std::string line;
        while(std::getline(pf, line)) {
            std::istringstream ls(line);
            std::string key; ls >> key;
            double v; std::vector<double> vals;
            while(ls >> v) vals.push_back(v);
            p[key] = vals;
        }
        auto wf = std::make_shared<Waveform>();
        wf->duration_ = (float)p.at("duration")[0];
        const auto& pu = p.at("pulse");
        for(std::size_t i = 0; i < (std::size_t)pu[0]; i++) wf->taps.emplace_back((float)pu[1 + 2 * i], (float)pu[2 + 2 * i]);
        auto beam = std::make_shared<BeamDirectivity>();
        beam->span_ = (float)p.at("beam_span")[0];
        for(std::size_t i = 0; i < (std::size_t)p.at("beam")[0]; i++) beam->values.push_back((float)p.at("beam")[1 + i]);
        auto info = std::make_shared<SensorInfo2D>();
        for(std::size_t i = 0; i < (std::size_t)p.at("bearings")[0]; i++) info->bearings_.push_back((float)p.at("bearings")[1 + i]);
        info->beam_ = beam;

        BoundSensorInstance2D s;
        s.ranges_ = Linspace<float>{(float)p.at("range_min")[0], (float)p.at("range_max")[0], (unsigned int)p.at("range_count")[0]};
        s.soundCelerity_ = (float)p.at("celerity")[0];
        s.waveform_ = wf;
        s.info_ = info;
        s.generate_psf_data_rtacx(argc > 4 && std::strcmp(argv[4], "texture") == 0 ? RTACX_FLAG_TEXTURE_PSF : 0u);

        std::ifstream sf(argv[2], std::ios::binary | std::ios::ate);
        const std::size_t bytes = (std::size_t)sf.tellg();
        sf.seekg(0);
        std::vector<SimSample2D> host(bytes / sizeof(SimSample2D));
        sf.read(reinterpret_cast<char*>(host.data()), (std::streamsize)(host.size() * sizeof(SimSample2D)));
        s.receivedSamples_.resize(host.size());
        if(cudaMemcpy(s.receivedSamples_.data(), host.data(), host.size() * sizeof(SimSample2D), cudaMemcpyHostToDevice) != cudaSuccess)
            throw std::runtime_error("copy of the samples failed");

        cuda::CudaPing2D<Complex<float>> ping;
        s.fill_ping_rtacx(ping, true);
        std::vector<Complex<float>> out(ping.ping_data_container().size());
        if(cudaMemcpy(out.data(), ping.ping_data_container().data(), out.size() * sizeof(Complex<float>), cudaMemcpyDeviceToHost) != cudaSuccess)
            throw std::runtime_error("copy of the ping failed");
        s.release_rtacx();
        std::ofstream of(argv[3], std::ios::binary);
        of.write(reinterpret_cast<const char*>(out.data()), (std::streamsize)(out.size() * sizeof(Complex<float>)));
        std::printf("margin %.9g\n", (double)(s.soundCelerity_ * wf->duration()));
    }
    catch(const std::exception& e) {
        std::cerr << "run_ping: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
