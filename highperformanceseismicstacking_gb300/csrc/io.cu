// io.cu -- result files written from a result slab in one pass per file.
//
// The reference writes each result (semblance, stack, every parameter) as an
// SU file with one trace per CDP: the CDP's 240-byte header, then its S
// samples, one ofstream write per header and per trace
// (Dumper::dumpResult, common/src/output/Dumper.cpp:77-114), from per-CDP
// vectors of the ResultSet (ResultSet.cpp:14-27).  Here a whole file image
// (nM0 x (240 + 4 S) bytes) is assembled in one host buffer -- the headers
// once, the samples of row r of every midpoint by one strided copy straight
// from the result slab [nM0][rows][S] (a 2-D copy from device memory when the
// slab is on the GPU) -- and written with one fwrite.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/hpss.h"
#include "hpss_internal.h"

namespace hpss {
void set_thread_error(const std::string &msg);
}  // namespace hpss

extern "C" hpss_status hpss_write_result_files(const float *slab, int slabOnDevice,
                                               uint32_t nM0, uint32_t rows, uint32_t S,
                                               const void *headers,
                                               const char *const *paths) {
    using hpss::set_thread_error;
    if (rows == 0 || nM0 == 0) return HPSS_OK;
    if (!slab || !headers || !paths || S == 0) {
        set_thread_error("null argument or S == 0");
        return HPSS_ERR_INVALID_ARGUMENT;
    }
    constexpr size_t kHeader = 240;  // sizeof(trace_info_t), Trace.hpp:9-91
    const size_t rec = kHeader + (size_t)S * sizeof(float);
    const size_t bytes = (size_t)nM0 * rec;
    // page-locked when the samples come from the device, so the strided copy
    // runs at full speed; pageable otherwise
    unsigned char *img = nullptr;
    std::vector<unsigned char> pageable;
    if (slabOnDevice) {
        cudaError_t e = cudaMallocHost(reinterpret_cast<void **>(&img), bytes);
        if (e != cudaSuccess) {
            set_thread_error(std::string("cudaMallocHost: ") + cudaGetErrorString(e));
            return HPSS_ERR_OUT_OF_MEMORY;
        }
    } else {
        pageable.resize(bytes);
        img = pageable.data();
    }
    const unsigned char *hdr = static_cast<const unsigned char *>(headers);
    for (uint32_t i = 0; i < nM0; i++) std::memcpy(img + i * rec, hdr + i * kHeader, kHeader);
    hpss_status rc = HPSS_OK;
    for (uint32_t r = 0; r < rows && rc == HPSS_OK; r++) {
        if (!paths[r]) continue;  // rows the caller does not want
        const float *src = slab + (size_t)r * S;
        if (slabOnDevice) {
            cudaError_t e = cudaMemcpy2D(img + kHeader, rec, src, (size_t)rows * S * sizeof(float),
                                         (size_t)S * sizeof(float), nM0, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) {
                set_thread_error(std::string("cudaMemcpy2D: ") + cudaGetErrorString(e));
                rc = HPSS_ERR_CUDA;
                break;
            }
        } else {
            for (uint32_t i = 0; i < nM0; i++)
                std::memcpy(img + i * rec + kHeader, src + (size_t)i * rows * S,
                            (size_t)S * sizeof(float));
        }
        FILE *f = std::fopen(paths[r], "wb");
        if (!f) {
            set_thread_error(std::string("Couldn't open ") + paths[r] +
                             " file to write result data.");
            rc = HPSS_ERR_INVALID_ARGUMENT;
            break;
        }
        const size_t wrote = std::fwrite(img, 1, bytes, f);
        if (std::fclose(f) != 0 || wrote != bytes) {
            set_thread_error(std::string("short write to ") + paths[r]);
            rc = HPSS_ERR_INVALID_ARGUMENT;
        }
    }
    if (slabOnDevice) cudaFreeHost(img);
    return rc;
}
