// nova-gb300: tensor-core belief scoring (placeholder until the tcgen05
// kernel lands; every update takes the exact path).

#include "pbvi.h"

namespace nova_gb300 {

__device__ unsigned int g_device_error = 0;

unsigned read_and_clear_device_error() {
    unsigned h = 0;
    if (cudaMemcpyFromSymbol(&h, g_device_error, sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (h != 0) {
        const unsigned zero = 0;
        cudaMemcpyToSymbol(g_device_error, &zero, sizeof(unsigned));
    }
    return h;
}

unsigned tc_device_error() { return 0; }

bool tc_supported(const DevModel &) { return false; }
int tc_build(BackupEngine &, const char *) { return NOVA_ERROR_INVALID_DATA; }
int tc_score(BackupEngine &, const float *, unsigned, unsigned *, const char *) { return NOVA_ERROR_INVALID_DATA; }
void tc_release(TcState *) {}

}  // namespace nova_gb300
