// genBasis of the IrradianceProbes facade (include/irradiance_probes.hpp)
// on the unit vectors read from stdin (float32 triples): writes b1 and b2 of
// each (six float32) to stdout.
#include <cstdio>

#include "irradiance_probes.hpp"

int main() {
    float n[3], b[6];
    while (std::fread(n, sizeof(float), 3, stdin) == 3) {
        ddgi::IrradianceProbes::genBasis(n, b, b + 3);
        std::fwrite(b, sizeof(float), 6, stdout);
    }
    return 0;
}
