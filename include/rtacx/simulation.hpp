// rtacx/simulation.hpp -- C++ host mirror of rtac_simulation's receiver API
// on top of the rtacx C ABI (rtacx.h).
//
// Same class names, argument meanings and error behaviour as the reference
// for the receiver path, so code written against the reference's
// SensorInstance reads the same:
//   Waveform_Sine        include/rtac_simulation/Waveform.h:96-138
//   BeamDirectivity      include/rtac_simulation/BeamDirectivity.h:52-104
//                        (a table + span; the reference's SincFunction table
//                        lives in non-vendored rtac_base)
//   SensorInfo(2D)       include/rtac_simulation/SensorInfo.h:18-104
//   SensorInstance1D_Complex / SensorInstance2D_Complex
//                        include/rtac_simulation/SensorInstance1D.h:72-110,
//                        include/rtac_simulation/SensorInstance2D.h:153-205
// set_ranges() re-derives the adaptive pulse duration, the Binner margin
// (c * duration) and the PSF tables exactly as SensorInstance::set_ranges
// (src/SensorInstance.cu:23-34); compute_output() runs sort + bin + reduce in
// one rtacx_reduce call on the legacy default stream and waits for it, as the
// reference does. Failures throw std::runtime_error with the library message.
// Device buffers use the CUDA runtime (cudaMalloc / cudaMemcpy), as
// rtac_base's CudaVector does.
#pragma once

#include <cmath>
#include <complex>
#include <cstdint>
#include <fstream>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../rtacx.h"

namespace rtacx { namespace simulation {

using Complex = std::complex<float>;

inline void check_cuda(cudaError_t e, const char* what)
{
    if(e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// rtac_base Linspace<float>: [lower, upper] sampled with `size` points.
struct Linspace {
    float lower_ = 0.0f, upper_ = 1.0f;
    unsigned int size_ = 2;
    Linspace() = default;
    Linspace(float l, float u, unsigned int n) : lower_(l), upper_(u), size_(n) {}
    float lower() const { return lower_; }
    float upper() const { return upper_; }
    unsigned int size() const { return size_; }
    float resolution() const { return (upper_ - lower_) / (size_ - 1); }
};

// Device array (rtac_base CudaVector stand-in).
template <typename T>
class DeviceVector {
    T* data_ = nullptr;
    std::size_t size_ = 0;
public:
    DeviceVector() = default;
    explicit DeviceVector(std::size_t n) { resize(n); }
    DeviceVector(const DeviceVector&) = delete;
    DeviceVector& operator=(const DeviceVector&) = delete;
    ~DeviceVector() { if(data_) cudaFree(data_); }
    void resize(std::size_t n)
    {
        if(n == size_) return;
        if(data_) cudaFree(data_);
        data_ = nullptr;
        size_ = n;
        if(n) check_cuda(cudaMalloc(&data_, n * sizeof(T)), "cudaMalloc");
    }
    std::size_t size() const { return size_; }
    T* data() { return data_; }
    const T* data() const { return data_; }
    void copy_from_host(const T* src, std::size_t n)
    {
        resize(n);
        if(n) check_cuda(cudaMemcpy(data_, src, n * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy");
    }
    std::vector<T> to_host() const
    {
        std::vector<T> out(size_);
        if(size_) check_cuda(cudaMemcpy(out.data(), data_, size_ * sizeof(T), cudaMemcpyDeviceToHost), "cudaMemcpy");
        return out;
    }
};

// Sample records (include/rtac_simulation/Sample.h:101-161).
struct SimSample1D { Complex value; float travel; };
struct SimSample2D { Complex value; float travel; float bearing; };
static_assert(sizeof(SimSample1D) == 12 && sizeof(SimSample2D) == 16, "sample layouts");

class Waveform {
public:
    using Ptr = std::shared_ptr<Waveform>;
    using ConstPtr = std::shared_ptr<const Waveform>;
    virtual ~Waveform() = default;
    bool fixed() const { return fixed_; }
    virtual void set_duration(float duration) = 0;
    virtual float duration() const = 0;
    virtual unsigned int size() const = 0;
    virtual Complex operator[](unsigned int idx) const = 0;
    virtual Ptr copy() const = 0;
protected:
    explicit Waveform(bool fixed) : fixed_(fixed) {}
    bool fixed_;
};

class Waveform_Sine : public Waveform {
    float frequency_, duration_;
    unsigned int oversampling_;
    Waveform_Sine(float f, float d, bool fixed, unsigned int os)
        : Waveform(fixed), frequency_(f), duration_(d), oversampling_(os) {}
public:
    static Ptr Create(float frequency, float duration, bool fixed, unsigned int oversampling = 8)
    {
        return Ptr(new Waveform_Sine(frequency, duration, fixed, oversampling));
    }
    void set_duration(float duration) override { if(!fixed()) duration_ = duration; }
    float sample_rate() const { return 2 * frequency_ * oversampling_; }
    float frequency() const { return frequency_; }
    float duration() const override { return duration_; }
    unsigned int size() const override { return this->sample_rate() * duration_; }
    Complex operator[](unsigned int idx) const override
    {
        const float phase = idx * (2.0 * M_PI * frequency_ / this->sample_rate());
        return Complex(std::cos(phase), std::sin(phase));
    }
    Ptr copy() const override { return Create(frequency_, duration_, fixed(), oversampling_); }
};

// A waveform given as a table whose duration follows the sensor.
class Waveform_Table : public Waveform {
    std::vector<Complex> taps_;
    float duration_;
    Waveform_Table(std::vector<Complex> taps, float d, bool fixed) : Waveform(fixed), taps_(std::move(taps)), duration_(d) {}
public:
    static Ptr Create(std::vector<Complex> taps, float duration, bool fixed)
    {
        return Ptr(new Waveform_Table(std::move(taps), duration, fixed));
    }
    void set_duration(float duration) override { if(!fixed()) duration_ = duration; }
    float duration() const override { return duration_; }
    unsigned int size() const override { return (unsigned int)taps_.size(); }
    Complex operator[](unsigned int idx) const override { return taps_[idx]; }
    Ptr copy() const override { return Create(taps_, duration_, fixed()); }
};

class BeamDirectivity {
    float span_;
    std::vector<float> data_;
    BeamDirectivity(float span, std::vector<float> data) : span_(span), data_(std::move(data)) {}
public:
    using Ptr = std::shared_ptr<BeamDirectivity>;
    using ConstPtr = std::shared_ptr<const BeamDirectivity>;
    static Ptr Create(float span, std::vector<float> data) { return Ptr(new BeamDirectivity(span, std::move(data))); }
    float span() const { return span_; }
    unsigned int size() const { return (unsigned int)data_.size(); }
    float operator[](unsigned int idx) const { return data_[idx]; }
    const std::vector<float>& data() const { return data_; }
};

class SensorInfo {
public:
    using Ptr = std::shared_ptr<SensorInfo>;
    using ConstPtr = std::shared_ptr<const SensorInfo>;
    virtual ~SensorInfo() = default;
    static Ptr Create(const Linspace& ranges, const Waveform::Ptr& waveform)
    {
        return Ptr(new SensorInfo(ranges, waveform));
    }
    const Linspace& ranges() const { return ranges_; }
    Waveform::ConstPtr waveform() const { return waveform_; }
protected:
    SensorInfo(const Linspace& ranges, const Waveform::Ptr& waveform)
        : ranges_(ranges), waveform_(waveform), soundCelerity_(1500.0f)
    {
        waveform_->set_duration(2 * ranges_.resolution() / soundCelerity_);   // SensorInfo.h:40
    }
    Linspace ranges_;
    Waveform::Ptr waveform_;
    float soundCelerity_;
};

class SensorInfo2D : public SensorInfo {
    std::vector<float> bearings_;
    BeamDirectivity::Ptr beam_;
    SensorInfo2D(std::vector<float> bearings, const Linspace& ranges, const Waveform::Ptr& waveform,
                 const BeamDirectivity::Ptr& beam)
        : SensorInfo(ranges, waveform), bearings_(std::move(bearings)), beam_(beam) {}
public:
    using Ptr = std::shared_ptr<SensorInfo2D>;
    using ConstPtr = std::shared_ptr<const SensorInfo2D>;
    static Ptr Create(std::vector<float> bearings, const Linspace& ranges, const Waveform::Ptr& waveform,
                      const BeamDirectivity::Ptr& beam)
    {
        return Ptr(new SensorInfo2D(std::move(bearings), ranges, waveform, beam));
    }
    const std::vector<float>& bearings() const { return bearings_; }
    BeamDirectivity::ConstPtr beam_directivity() const { return beam_; }
    unsigned int width() const { return (unsigned int)bearings_.size(); }
    unsigned int height() const { return ranges_.size(); }
};

// Owns one rtacx context; shared by the 1D and 2D instances.
class SensorInstance {
public:
    virtual ~SensorInstance() { rtacx_destroy(ctx_); }
    const Linspace& ranges() const { return ranges_; }
    Waveform::ConstPtr waveform() const { return waveform_; }
    float sound_celerity() const { return soundCelerity_; }

    void set_ranges(const Linspace& ranges, float soundCelerity)
    {
        soundCelerity_ = soundCelerity;
        this->set_ranges(ranges);
    }
    void set_ranges(const Linspace& ranges)       // src/SensorInstance.cu:23-34
    {
        ranges_ = ranges;
        if(!waveform_->fixed()) waveform_->set_duration(ranges.resolution() / soundCelerity_);
        this->configure();
    }
    void set_ranges(float maxRange, unsigned int rangeCount)
    {
        this->set_ranges(Linspace(ranges_.lower(), maxRange, rangeCount));
    }
    virtual void set_sample_count(unsigned int count) = 0;
    virtual unsigned int sample_count() const = 0;
    virtual void compute_output() = 0;

protected:
    SensorInstance(const Linspace& ranges, const Waveform::ConstPtr& waveform, float soundCelerity)
        : ranges_(ranges), waveform_(waveform->copy()), soundCelerity_(soundCelerity)
    {
        const rtacx_status st = rtacx_create(&ctx_, 0);
        if(st != RTACX_OK)
            throw std::runtime_error("rtacx: cannot create a context on CUDA device 0 (status " +
                                     std::to_string((int)st) + ")");
    }
    void check(rtacx_status st) const
    {
        if(st != RTACX_OK)
            throw std::runtime_error(std::string("rtacx: ") + rtacx_last_error(ctx_) + " (status " +
                                     std::to_string((int)st) + ")");
    }
    std::vector<Complex> pulse_table() const
    {
        std::vector<Complex> p(waveform_->size());
        for(unsigned int i = 0; i < p.size(); i++) p[i] = (*waveform_)[i];
        return p;
    }
    float margin() const { return soundCelerity_ * waveform_->duration(); }   // Binner margin
    virtual void configure() = 0;

    rtacx_ctx* ctx_ = nullptr;
    Linspace ranges_;
    Waveform::Ptr waveform_;
    float soundCelerity_;
};

class SensorInstance1D_Complex : public SensorInstance {
    DeviceVector<SimSample1D> receivedSamples_;
    DeviceVector<Complex> sensorOutput_;
    SensorInstance1D_Complex(const SensorInfo::ConstPtr& info, float c)
        : SensorInstance(info->ranges(), info->waveform(), c)
    {
        this->set_ranges(info->ranges());
    }
    void configure() override
    {
        const std::vector<Complex> pulse = pulse_table();
        rtacx_sensor_1d s{};
        s.range_min = ranges_.lower(); s.range_max = ranges_.upper(); s.range_count = ranges_.size();
        s.sound_celerity = soundCelerity_; s.pulse_duration = waveform_->duration(); s.margin = margin();
        s.pulse = reinterpret_cast<const float*>(pulse.data()); s.pulse_len = (uint32_t)pulse.size();
        check(rtacx_configure_1d(ctx_, &s));
    }
public:
    using Ptr = std::shared_ptr<SensorInstance1D_Complex>;
    static Ptr Create(const SensorInfo::ConstPtr& info, float soundCelerity = 1500.0f)
    {
        return Ptr(new SensorInstance1D_Complex(info, soundCelerity));
    }
    unsigned int size() const { return ranges_.size(); }
    void set_sample_count(unsigned int count) override { receivedSamples_.resize(count); }
    unsigned int sample_count() const override { return (unsigned int)receivedSamples_.size(); }
    DeviceVector<SimSample1D>& samples() { return receivedSamples_; }
    const DeviceVector<Complex>& output() const { return sensorOutput_; }
    void compute_output() override
    {
        sensorOutput_.resize(this->size());
        check(rtacx_reduce(ctx_, receivedSamples_.data(), receivedSamples_.size(),
                           reinterpret_cast<float*>(sensorOutput_.data()), nullptr));
        check(rtacx_stream_status(ctx_, nullptr));
    }
};

class SensorInstance2D_Complex : public SensorInstance {
    SensorInfo2D::ConstPtr info_;
    DeviceVector<SimSample2D> receivedSamples_;
    DeviceVector<Complex> sensorOutput_;
    bool texturePsf_ = false;
protected:
    SensorInstance2D_Complex(const SensorInfo2D::ConstPtr& info, float c)
        : SensorInstance(info->ranges(), info->waveform(), c), info_(info)
    {
        this->set_ranges(info->ranges());
    }
private:
    void configure() override
    {
        const std::vector<Complex> pulse = pulse_table();
        const auto& beam = *info_->beam_directivity();
        rtacx_sensor_2d s{};
        s.range_min = ranges_.lower(); s.range_max = ranges_.upper(); s.range_count = ranges_.size();
        s.sound_celerity = soundCelerity_; s.pulse_duration = waveform_->duration(); s.margin = margin();
        s.pulse = reinterpret_cast<const float*>(pulse.data()); s.pulse_len = (uint32_t)pulse.size();
        s.beam = beam.data().data(); s.beam_len = beam.size(); s.beam_span = beam.span();
        s.bearings = info_->bearings().data(); s.bearing_count = (uint32_t)info_->bearings().size();
        s.flags = texturePsf_ ? RTACX_FLAG_TEXTURE_PSF : 0u;
        check(rtacx_configure_2d(ctx_, &s));
    }
public:
    using Ptr = std::shared_ptr<SensorInstance2D_Complex>;
    // Evaluate the PSF on the texture unit as the reference's
    // SensorInstance2D does (RTACX_FLAG_TEXTURE_PSF): the ping then matches
    // the reference's own to float round-off. Off: exact bilinear weights.
    void set_texture_psf(bool on)
    {
        texturePsf_ = on;
        this->set_ranges(ranges_);
    }
    static Ptr Create(const SensorInfo2D::ConstPtr& info, float soundCelerity = 1500.0f)
    {
        return Ptr(new SensorInstance2D_Complex(info, soundCelerity));
    }
    static Ptr Create(const SensorInfo::ConstPtr& info, float soundCelerity = 1500.0f)
    {
        auto info2d = std::dynamic_pointer_cast<const SensorInfo2D>(info);
        if(!info2d) throw std::runtime_error("A SensorInstance2D must be created with a SensorInfo2D instance");
        return Create(info2d, soundCelerity);
    }
    unsigned int width() const { return info_->width(); }
    unsigned int height() const { return ranges_.size(); }
    unsigned int size() const { return this->width() * this->height(); }
    const std::vector<float>& bearings() const { return info_->bearings(); }
    void set_sample_count(unsigned int count) override { receivedSamples_.resize(count); }
    unsigned int sample_count() const override { return (unsigned int)receivedSamples_.size(); }
    DeviceVector<SimSample2D>& samples() { return receivedSamples_; }
    const DeviceVector<Complex>& output() const { return sensorOutput_; }
    void compute_output() override
    {
        sensorOutput_.resize(this->size());
        check(rtacx_reduce(ctx_, receivedSamples_.data(), receivedSamples_.size(),
                           reinterpret_cast<float*>(sensorOutput_.data()), nullptr));
        check(rtacx_stream_status(ctx_, nullptr));
    }
};

// A device ping with its geometry: the counterpart of rtac_base's
// cuda::CudaPing2D<Complex<float>> as returned by the reference's
// SensorInstance2D_2<T>::get_ping() (include/rtac_simulation/SensorInstance2D.h:144):
// range Linspace, bearings, [range][bearing] complex64 data on the device.
class Ping2D {
    Linspace ranges_;
    std::vector<float> bearings_;
    const Complex* data_;
public:
    Ping2D(const Linspace& ranges, std::vector<float> bearings, const Complex* data)
        : ranges_(ranges), bearings_(std::move(bearings)), data_(data) {}
    const Linspace& ranges() const { return ranges_; }
    const std::vector<float>& bearings() const { return bearings_; }
    unsigned int width() const { return (unsigned int)bearings_.size(); }
    unsigned int height() const { return ranges_.size(); }
    unsigned int size() const { return width() * height(); }
    const Complex* ping_data() const { return data_; }
    std::vector<Complex> to_host() const
    {
        std::vector<Complex> out(size());
        if(!out.empty())
            check_cuda(cudaMemcpy(out.data(), data_, out.size() * sizeof(Complex), cudaMemcpyDeviceToHost), "cudaMemcpy");
        return out;
    }
};

// The reference's scalar-templated 2D instance
// (include/rtac_simulation/SensorInstance2D.h:96-151), which its factory
// creates as SensorInstance2D_2<Complex<float>> (src/factories/SensorInfoFactory.cpp:28).
// The reference reduces into complex pings only (src/SensorInstance2D.cu:85-119),
// so Complex is the only supported scalar. The receiver pose of the
// reference's Create() belongs to the ray caster and is not modelled here.
template <typename T>
class SensorInstance2D_2 {
    static_assert(sizeof(T) == 0, "SensorInstance2D_2 supports Complex pings only, as the reference's do_reduce");
};

template <>
class SensorInstance2D_2<Complex> : public SensorInstance2D_Complex {
    SensorInstance2D_2(const SensorInfo2D::ConstPtr& info, float c) : SensorInstance2D_Complex(info, c) {}
public:
    using Ptr = std::shared_ptr<SensorInstance2D_2<Complex>>;
    static Ptr Create(const SensorInfo2D::ConstPtr& info, float soundCelerity = 1500.0f)
    {
        return Ptr(new SensorInstance2D_2<Complex>(info, soundCelerity));
    }
    static Ptr Create(const SensorInfo::ConstPtr& info, float soundCelerity = 1500.0f)
    {
        auto info2d = std::dynamic_pointer_cast<const SensorInfo2D>(info);
        if(!info2d) throw std::runtime_error("A SensorInstance2D must be created with a SensorInfo2D instance");
        return Create(info2d, soundCelerity);
    }
    bool is_complex() const { return true; }
    Ping2D get_ping() const { return Ping2D(this->ranges(), this->bearings(), this->output().data()); }
};

// Ping file sink (include/rtac_simulation/sinks/FileSink.h:15-37,
// src/sinks/FileSink.cpp:14-42): appends one record per set_output() call.
// The reference serialises rtac_base's CudaPing2D, whose wire format lives in
// the non-vendored rtac_base serialization; this sink writes its own
// documented little-endian record instead:
//   char magic[8] = "RTACXPNG"; uint32 version = 1; uint32 range_count;
//   uint32 bearing_count; float range_min, range_max;
//   float bearings[bearing_count]; complex64 ping[range_count][bearing_count]
// Like the reference, only 2D sensors are written.
class FileSink {
    std::string filename_;
    std::ofstream* file_;
    explicit FileSink(const std::string& filename)
        : filename_(filename), file_(new std::ofstream(filename, std::ofstream::binary)) {}
public:
    using Ptr = std::shared_ptr<FileSink>;
    ~FileSink() { delete file_; }
    static Ptr Create(const std::string& filename, bool overwrite = false)
    {
        std::ifstream probe(filename);
        if(probe.good() && !overwrite)
            throw std::runtime_error("FileSink : could not prepare path for file '" + filename + "'");
        Ptr p(new FileSink(filename));
        if(!p->file_->good()) throw std::runtime_error("FileSink : cannot open '" + filename + "'");
        return p;
    }
    const std::string& filename() const { return filename_; }
    void set_output(const std::shared_ptr<SensorInstance2D_Complex>& sensor)
    {
        if(!sensor) { std::cerr << "FileSink : sensor type not handled" << std::endl; return; }
        const std::vector<Complex> ping = sensor->output().to_host();
        const uint32_t version = 1, nr = sensor->height(), nb = sensor->width();
        const float rmin = sensor->ranges().lower(), rmax = sensor->ranges().upper();
        file_->write("RTACXPNG", 8);
        file_->write(reinterpret_cast<const char*>(&version), 4);
        file_->write(reinterpret_cast<const char*>(&nr), 4);
        file_->write(reinterpret_cast<const char*>(&nb), 4);
        file_->write(reinterpret_cast<const char*>(&rmin), 4);
        file_->write(reinterpret_cast<const char*>(&rmax), 4);
        file_->write(reinterpret_cast<const char*>(sensor->bearings().data()), 4 * (std::streamsize)nb);
        file_->write(reinterpret_cast<const char*>(ping.data()), (std::streamsize)(ping.size() * sizeof(Complex)));
        file_->flush();
        if(!file_->good()) throw std::runtime_error("FileSink : write failed on '" + filename_ + "'");
    }
};

}} // namespace rtacx::simulation
