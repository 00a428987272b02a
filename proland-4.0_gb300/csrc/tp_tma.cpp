// TMA tensor-map descriptors over tile pools.  The driver entry point is looked
// up at run time through the CUDA runtime, so the library does not link libcuda.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstring>

#include "tp_internal.h"
#include "tp_learned.h"

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn(int *err)
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    static cudaError_t status = cudaSuccess;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        status = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (status == cudaSuccess && q == cudaDriverEntryPointSuccess) fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    if (!fn) *err = tp::fail(TP_E_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    return fn;
}

}  // namespace

namespace tp {

int tensor_map(tp_storage *s, int box_x, int box_y, const CUtensorMap **out)
{
    auto key = std::make_pair(box_x, box_y);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->maps.find(key);
        if (it != s->maps.end()) {
            *out = &it->second;
            return TP_OK;
        }
    }
    if (box_x < 1 || box_x > 256 || box_y < 1 || box_y > 256 || (box_x * 4) % 16 != 0)
        return fail(TP_E_BAD_ARG, "tensor map: box outside TMA limits");
    int err = TP_OK;
    auto fn = encode_fn(&err);
    if (!fn) return err;
    CUtensorMap m;
    std::memset(&m, 0, sizeof m);
    cuuint64_t dims[3] = {(cuuint64_t)s->W, (cuuint64_t)s->W, (cuuint64_t)s->capacity * s->channels};
    cuuint64_t strides[2] = {(cuuint64_t)s->pitch * sizeof(float), (cuuint64_t)s->plane_stride * sizeof(float)};
    cuuint32_t box[3] = {(cuuint32_t)box_x, (cuuint32_t)box_y, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, s->base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(TP_E_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    std::lock_guard<std::mutex> lk(s->mu);
    auto ins = s->maps.emplace(key, m);
    *out = &ins.first->second;
    return TP_OK;
}

int encode_tensor_map(const tp_storage *s, int box_x, int box_y, CUtensorMap *out)
{
    if (box_x < 1 || box_x > 256 || box_y < 1 || box_y > 256 || (box_x * 4) % 16 != 0)
        return fail(TP_E_BAD_ARG, "tensor map: box outside TMA limits");
    int err = TP_OK;
    auto fn = encode_fn(&err);
    if (!fn) return err;
    std::memset(out, 0, sizeof *out);
    cuuint64_t dims[3] = {(cuuint64_t)s->W, (cuuint64_t)s->W, (cuuint64_t)s->capacity * s->channels};
    cuuint64_t strides[2] = {(cuuint64_t)s->pitch * sizeof(float), (cuuint64_t)s->plane_stride * sizeof(float)};
    cuuint32_t box[3] = {(cuuint32_t)box_x, (cuuint32_t)box_y, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, s->base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(TP_E_CUDA, "cuTensorMapEncodeTiled failed");
    return TP_OK;
}

}  // namespace tp

namespace tp {
namespace learned {

// bf16 activations of `nimg` images of (W+2)^2 pixels, stored as channels / 8
// planes per image of 16-byte pixels (8 channels), seen as a 3D tensor (x and
// channel merged: (W+2) x 8 elements per row, y, image x group); boxes of box_x
// whole pixels (box_x x 16 contiguous bytes) x box_y rows of one plane; reads
// outside the tensor return zeros.
int encode_act_map(void *base, int W, int channels, int nimg, int box_x, int box_y, CUtensorMap *out)
{
    if (channels % 8 != 0 || box_x < 1 || box_x > 32 || box_y < 1 || box_y > 256 || nimg < 1)
        return fail(TP_E_BAD_ARG, "activation tensor map: bad shape");
    int err = TP_OK;
    auto fn = encode_fn(&err);
    if (!fn) return err;
    std::memset(out, 0, sizeof *out);
    const cuuint64_t Wp = (cuuint64_t)W + 2;
    cuuint64_t dims[3] = {Wp * 8, Wp, (cuuint64_t)nimg * (channels / 8)};
    cuuint64_t strides[2] = {Wp * 16, Wp * Wp * 16};
    cuuint32_t box[3] = {(cuuint32_t)box_x * 8, (cuuint32_t)box_y, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(out, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(TP_E_CUDA, "cuTensorMapEncodeTiled failed (activations)");
    return TP_OK;
}

}  // namespace learned
}  // namespace tp
