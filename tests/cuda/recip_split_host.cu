// Host side of the division by a per-scene constant (tss_device.cuh): prints, for
// each divisor b given on standard input (one float per line, %a or decimal),
// "b yh yl" as hexadecimal floats, where recip_split(b) = (yh, yl).  Runs on any
// machine (no CUDA call).
#include <cstdio>
#include <cstdlib>

#include "../../twoscalesplit_gb300/csrc/tss_device.cuh"

int main() {
    char line[128];
    while (std::fgets(line, sizeof line, stdin)) {
        const float b = std::strtof(line, nullptr);
        float yh = 0.0f, yl = 0.0f;
        tss::recip_split(b, yh, yl);
        std::printf("%a %a %a\n", b, yh, yl);
    }
    return 0;
}
