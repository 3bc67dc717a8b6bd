// qp3d_noalloc.cu -- max|grad u| of a caller's device wavefield without any
// device allocation.
//
// Some callers cannot let a library allocate device memory: a host program
// whose framework has already reserved the whole device for its own pool, or
// a real-time loop that forbids allocation after start-up.
// qp3d_gradmax_noalloc serves them.  It is the gradmax kernel of the
// library, with its scratch (one partial maximum per CTA and an error word)
// in file-scope device arrays of this translation unit instead of buffers
// the library allocates; the caller passes the wavefield and the output
// location.
//
// The arrays exist once per device that loads the library and are held until
// the process exits.  Every call shares them and they keep the last call's
// contents, so calls that overlap on the GPU (different streams, or host
// threads without ordering) race.  Each call clears the error word before it
// launches; every partial slot it reads is written by the same call.  The
// call waits for its stream before it returns, so that a bounded device wait
// that ran out is reported as QP3D_ERR_TIMEOUT.
#include "qp3d.h"
#include "qp3d_internal.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace qp3d {
void derive_coefs(const float *c, const float *c2, float dx, float dy, float dz, Coefs *k);
}
using namespace qp3d;

namespace {

// Largest grid the partial array holds: one float per CTA (256 KB).  With
// 32-cell x 32-row tiles this covers nx*ny up to about 64 M cells per plane.
constexpr unsigned kNoAllocMaxBlocks = 1u << 16;

static __device__ __align__(256) float g_noalloc_partial[kNoAllocMaxBlocks];
static __device__ __align__(256) unsigned g_noalloc_err[64];

struct DeviceScratch {
    bool ready;
    float *partial;
    unsigned *err;
};
constexpr int kMaxDevices = 64;
DeviceScratch g_dev[kMaxDevices];
std::mutex g_mutex;

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn g_encode = nullptr;

int report(char *err, size_t errlen, int code, const char *msg)
{
    if (err && errlen) snprintf(err, errlen, "%s", msg);
    return code;
}

// test hooks (set through qp3d_tune with a NULL context)
unsigned long long g_wait_ns = 0;   // 0: the kernels' default (2 s)
int g_hold_plane = 0;               // withheld plane + 1 in the first CTA, 0: none

}  // namespace

namespace qp3d {
int noalloc_tune(const char *key, int value)
{
    if (!strcmp(key, "noalloc_wait_limit_us") && value >= 0) g_wait_ns = 1000ull * (unsigned)value;
    else if (!strcmp(key, "noalloc_test_hold_plane") && value >= -1) g_hold_plane = value + 1;
    else return QP3D_ERR_ARG;
    return QP3D_OK;
}
}  // namespace qp3d

extern "C" int qp3d_gradmax_noalloc(const float *d_u, int nx, int ny, int nz, int ldy, float dx,
                                    float dy, float dz, const float *c, float *d_max,
                                    void *stream, char *err, size_t errlen)
{
    char msg[256];
    if (err && errlen) err[0] = 0;
    if (!d_u || !d_max || !c)
        return report(err, errlen, QP3D_ERR_ARG, "null wavefield, output or coefficient table");
    if (nx < 11 || ny < 11 || nz < 11)
        return report(err, errlen, QP3D_ERR_ARG, "grid smaller than 11 cells in some direction");
    if (ldy < ny || ldy % 4 != 0)
        return report(err, errlen, QP3D_ERR_ARG, "row pitch ldy must be >= ny and a multiple of 4");
    if (reinterpret_cast<uintptr_t>(d_u) % 16 != 0)
        return report(err, errlen, QP3D_ERR_ARG, "wavefield pointer must be 16-byte aligned");
    if (!(dx > 0) || !(dy > 0) || !(dz > 0))
        return report(err, errlen, QP3D_ERR_ARG, "non-positive spacing");

    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return report(err, errlen, QP3D_ERR_CUDA, "no usable CUDA device");

    // launch plan (as the shot path plans it)
    const int ncx = nx - 2 * kRadius, ncz = nz - 2 * kRadius;
    const int ntx = (ncx + kMaxTileX - 1) / kMaxTileX;
    const int tile_x = (ncx + ntx - 1) / ntx;
    const int nxt = (ncx + tile_x - 1) / tile_x;
    const int nyt = (ny - kRadius - 1) / kTileY + 1;
    const long long tiles = (long long)nxt * nyt;
    if (tiles > kNoAllocMaxBlocks) {
        snprintf(msg, sizeof(msg),
                 "grid %dx%d needs %lld tiles per z chunk; qp3d_gradmax_noalloc holds at most %u",
                 nx, ny, tiles, kNoAllocMaxBlocks);
        return report(err, errlen, QP3D_ERR_ARG, msg);
    }
    long long nch = (6ll * nsm + tiles - 1) / tiles;
    nch = std::max(1ll, std::min(nch, (long long)std::max(1, ncz / 24)));
    nch = std::min(nch, (long long)(kNoAllocMaxBlocks / tiles));
    const int chunk_z = (int)((ncz + nch - 1) / nch);
    nch = (ncz + chunk_z - 1) / chunk_z;
    // the launch grid is (y tiles, x tiles, z chunks); CUDA limits its second
    // and third dimensions to 65535
    if (nxt > 65535 || nch > 65535) {
        snprintf(msg, sizeof(msg),
                 "grid %dx%dx%d needs %d x tiles and %lld z chunks; the launch allows at most 65535",
                 nx, ny, nz, nxt, nch);
        return report(err, errlen, QP3D_ERR_ARG, msg);
    }
    const unsigned nblocks = (unsigned)(tiles * nch);

    // once per device, with that device current: the scratch addresses and
    // the kernel's shared-memory limit.  The first call on a device does this
    // set-up; make it before any stream capture.
    DeviceScratch ds;
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        if (!g_encode) {
            void *fn = nullptr;
            cudaDriverEntryPointQueryResult qr;
            if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                 cudaEnableDefault, &qr) != cudaSuccess ||
                qr != cudaDriverEntryPointSuccess || !fn)
                return report(err, errlen, QP3D_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
            g_encode = reinterpret_cast<EncodeTiledFn>(fn);
        }
        DeviceScratch &d = g_dev[dev];
        if (!d.ready) {
            float *pp = nullptr;
            unsigned *pe = nullptr;
            cudaError_t e1 = cudaGetSymbolAddress((void **)&pp, g_noalloc_partial);
            cudaError_t e2 = cudaGetSymbolAddress((void **)&pe, g_noalloc_err);
            if (e1 != cudaSuccess || e2 != cudaSuccess || !pp || !pe)
                return report(err, errlen, QP3D_ERR_CUDA, "cudaGetSymbolAddress failed");
            if (configure_gradmax_partial() != cudaSuccess)
                return report(err, errlen, QP3D_ERR_CUDA, "cannot set the kernel's shared memory");
            d.partial = pp;
            d.err = pe;
            d.ready = true;
        }
        ds = d;
    }

    CUtensorMap tm;
    cuuint64_t dims[3] = {(cuuint64_t)ny, (cuuint64_t)nx, (cuuint64_t)nz};
    cuuint64_t strides[2] = {(cuuint64_t)ldy * 4, (cuuint64_t)ldy * 4 * nx};
    cuuint32_t box[3] = {(cuuint32_t)kBoxY, (cuuint32_t)(tile_x + 2 * kRadius), 1};
    cuuint32_t es[3] = {1, 1, 1};
    if (g_encode(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(d_u), dims, strides,
                 box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                 CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return report(err, errlen, QP3D_ERR_CUDA, "cuTensorMapEncodeTiled failed");

    PlaneParams p;
    memset(&p, 0, sizeof(p));
    p.nx = nx; p.ny = ny; p.nz = nz; p.ldy = ldy; p.pml = 0; p.sz = 0;
    p.tile_x = tile_x;
    p.chunk_z = chunk_z;
    p.plane = (long long)nx * ldy;
    derive_coefs(c, c, dx, dy, dz, &p.k);   // first-derivative weights only
    p.arith = kArithFast;   // the library's default arithmetic
    p.err = ds.err;
    p.wait_ns = g_wait_ns;
    p.hold_plane = g_hold_plane;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the error word must start at zero; the partial slots are all written
    if (cudaMemsetAsync(ds.err, 0, sizeof(unsigned), s) != cudaSuccess)
        return report(err, errlen, QP3D_ERR_CUDA, "cannot clear the error word");
    dim3 grid(nyt, nxt, (unsigned)nch);
    cudaError_t e = launch_gradmax_partial(tm, p, grid, plane_smem_bytes(tile_x, 0), s, ds.partial,
                                           nblocks, d_max);
    if (e != cudaSuccess) {
        snprintf(msg, sizeof(msg), "launch failed: %s", cudaGetErrorString(e));
        return report(err, errlen, QP3D_ERR_CUDA, msg);
    }
    // wait for the result and report a device wait that ran out (d_max then
    // holds NaN); the error word is read into host memory, nothing allocated
    unsigned flags = 0;
    if ((e = cudaMemcpyAsync(&flags, ds.err, sizeof(unsigned), cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) {
        snprintf(msg, sizeof(msg), "%s", cudaGetErrorString(e));
        return report(err, errlen, QP3D_ERR_CUDA, msg);
    }
    if (flags) return report(err, errlen, QP3D_ERR_TIMEOUT, "a device wait timed out");
    return QP3D_OK;
}
