// settings_roundtrip.cpp - reads a settings file of the reference (or of this
// library) into the C++ mirror of taa<CF> and writes the mirror's settings
// back out, as the reference's loadSettings/saveSettings do around
// taa::readSettingsFromIni / writeSettingsToIni (source/main.cpp:4378, 4467).
//
//   settings_roundtrip <in.ini>      prints the settings file the mirror writes
// No device work: the mirror's settings live on the host.
#include <cstdio>
#include <fstream>
#include <sstream>

#include "../taa.hpp"

int main(int argc, char** argv) {
    taa_gb300::taa<3> taa;
    if (argc > 1) {
        std::ifstream f(argv[1], std::ios::binary);
        if (!f) {
            std::fprintf(stderr, "cannot open %s\n", argv[1]);
            return 1;
        }
        std::stringstream ss;
        ss << f.rdbuf();
        try {
            taa.readSettingsFromIni(ss.str());
        } catch (const std::exception& e) {
            std::fprintf(stderr, "%s\n", e.what());
            return 2;
        }
    }
    std::fputs(taa.writeSettingsToIni().c_str(), stdout);
    return 0;
}
