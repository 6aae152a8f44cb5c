// Golden-vector probe: compiles the reference's own header-only arithmetic
// (rtac_simulation/Binner.h Binner::Key, rtac_simulation/Waveform.h
// Waveform_Sine) against the host stand-ins in ref_stubs/ and prints its
// results with exact hexadecimal floats. Test infrastructure only: it is built
// by ref_build.sh into oracle/_ref/ and run by tests/golden/make_golden.py.
//
// Protocol (one request per stdin line, one answer per stdout line):
//   KEY nBins minBin maxBin margin n t_1 .. t_n
//     -> KEY a b lower upper k_1 .. k_n      (k_i = "x" where the float->int
//        conversion of fmaf(a, t, b) is outside int range or NaN: the host
//        conversion is undefined there, the device one saturates)
//   WAVE frequency duration oversampling
//     -> WAVE size re_0 im_0 .. re_{size-1} im_{size-1}
//   RECT width height wavelength baffle oversampling   (Directivity::rectangle_antenna)
//   DISK diameter wavelength baffle oversampling        (Directivity::disk_antenna)
//     -> DIR width height v_0 .. v_{w*h-1}   (row-major [h][w]; baffle: none | single-sided)
// Floats on input are parsed with strtof (hex or decimal); output uses %a.
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include <rtac_simulation/Binner.h>
#include <rtac_simulation/Waveform.h>
#include <rtac_simulation/Directivity.h>

using rtac::simulation::Binner;
using rtac::simulation::SimSample1D;
using rtac::simulation::Waveform_Sine;

static float parse_f(const std::string& s) { return std::strtof(s.c_str(), nullptr); }

int main()
{
    std::string line;
    while(std::getline(std::cin, line)) {
        std::istringstream in(line);
        std::string cmd; in >> cmd;
        if(cmd == "KEY") {
            std::string tok;
            unsigned int nBins; in >> nBins;
            in >> tok; float minBin = parse_f(tok);
            in >> tok; float maxBin = parse_f(tok);
            in >> tok; float margin = parse_f(tok);
            unsigned long n; in >> n;
            Binner::Key key(nBins, minBin, maxBin, margin);
            std::printf("KEY %a %a %a %a", key.a_, key.b_, key.bounds_.lower, key.bounds_.upper);
            for(unsigned long i = 0; i < n; i++) {
                in >> tok; float t = parse_f(tok);
                float f = std::fmaf(key.a_, t, key.b_);
                if(!(std::fabs(f) < 2.0e9f)) { std::printf(" x"); continue; }
                SimSample1D s = SimSample1D::Null();
                s.travel() = t;
                std::printf(" %u", key(s));
            }
            std::printf("\n");
        }
        else if(cmd == "WAVE") {
            std::string tok;
            in >> tok; float frequency = parse_f(tok);
            in >> tok; float duration  = parse_f(tok);
            unsigned int os; in >> os;
            auto w = Waveform_Sine::Create(frequency, duration, false, os);
            std::printf("WAVE %u", w->size());
            for(unsigned int i = 0; i < w->size(); i++) {
                auto v = (*w)[i];
                std::printf(" %a %a", v.real(), v.imag());
            }
            std::printf("\n");
        }
        else if(cmd == "RECT" || cmd == "DISK") {
            std::string tok, baffle;
            rtac::simulation::Directivity::Ptr d;
            if(cmd == "RECT") {
                in >> tok; float w = parse_f(tok);
                in >> tok; float h = parse_f(tok);
                in >> tok; float l = parse_f(tok);
                in >> baffle; unsigned int os; in >> os;
                d = rtac::simulation::Directivity::rectangle_antenna(w, h, l, baffle, os);
            }
            else {
                in >> tok; float dia = parse_f(tok);
                in >> tok; float l = parse_f(tok);
                in >> baffle; unsigned int os; in >> os;
                d = rtac::simulation::Directivity::disk_antenna(dia, l, baffle, os);
            }
            const auto& t = d->texture();
            std::printf("DIR %u %u", t.width, t.height);
            for(float v : t.image) std::printf(" %a", v);
            std::printf("\n");
        }
        std::fflush(stdout);
    }
    return 0;
}
