/*
 * xg_noalloc.cuh -- xin_gpu_fdct2_wxh_noalloc: the forward 2-D DCT2 of one
 * block held in device memory, for callers that must not allocate.
 *
 * Who needs it: code that runs where a cudaMalloc is not allowed or not
 * wanted -- a host thread with a real-time deadline (cudaMalloc can
 * synchronise the device), a caller in the middle of recording a CUDA graph,
 * or a caller whose memory budget is fixed up front.  The other per-call
 * forms allocate per-thread staging on first use; this one allocates nothing:
 * the caller passes device inputs and outputs, and the intermediate between
 * the two 1-D passes lives in a file-scope device array that every GPU
 * loading the library holds until exit.
 *
 * Limits and sharing: at most 64 x 64 coefficients per call.  All calls share
 * the one array and it keeps the last call's contents; every element a call
 * reads is written earlier by the same call, so nothing needs clearing.  Calls
 * that overlap on the GPU (two streams, two host threads) race on the array
 * and must be serialised by the caller.
 */

#define XG_NOALLOC_MAX_COEFFS (64 * 64)

static __device__ __align__(256) xg_coef g_noalloc_fdct_scratch[XG_NOALLOC_MAX_COEFFS];

/* device address of the scratch array, looked up once per device with that
 * device current (the host-side symbol is not a device address).  The lookup
 * is refused while `st` is capturing: make the first call on a device outside
 * any stream capture. */
static xg_coef *xg_noalloc_scratch(int dev, cudaStream_t st)
{
    static std::mutex mu;
    static xg_coef *ptr[64] = {};
    if (dev < 0 || dev >= 64) { xg_set_error(XIN_GPU_ERR_ARG, "noalloc: device index %d out of range", dev); return nullptr; }
    std::lock_guard<std::mutex> lock(mu);
    if (!ptr[dev]) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (xg_cuda_check(cudaStreamIsCapturing(st, &cs), "noalloc: cudaStreamIsCapturing")) return nullptr;
        if (cs != cudaStreamCaptureStatusNone) {
            xg_set_error(XIN_GPU_ERR_STATE, "fdct2_wxh_noalloc: the first call on device %d must come before any stream capture", dev);
            return nullptr;
        }
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_fdct_scratch);
        if (e != cudaSuccess) { xg_cuda_check(e, "noalloc: cudaGetSymbolAddress"); return nullptr; }
        ptr[dev] = (xg_coef *)p;
    }
    return ptr[dev];
}

extern "C" int xin_gpu_fdct2_wxh_noalloc(const XG_COEFF *input, intptr_t inputStride, XG_COEFF *output, intptr_t outputStride,
                                          uint32_t width, uint32_t height, int32_t shift1st, int32_t shift2nd, void *stream)
{
    xin_gpu_clear_error();
    int lw = xg_lg(width), lh = xg_lg(height);
    if (!input || !output || lw < 1 || lh < 1 || inputStride < (intptr_t)width || outputStride < (intptr_t)width) {
        xg_set_error(XIN_GPU_ERR_ARG, "fdct2_wxh_noalloc: null pointer, bad stride or size not a power of two >= 2");
        return XIN_GPU_ERR_ARG;
    }
    if ((size_t)width * height > XG_NOALLOC_MAX_COEFFS || lw > 6 || lh > 6) {
        xg_set_error(XIN_GPU_ERR_ARG, "fdct2_wxh_noalloc: %ux%u exceeds the 64x64 (%d-coefficient) scratch of this entry point",
                     width, height, XG_NOALLOC_MAX_COEFFS);
        return XIN_GPU_ERR_ARG;
    }
    /* no implicit initialisation here: it would make the library's device current
     * on the caller's thread, whose buffers may live on another device */
    if (g_init_status != XIN_GPU_OK) {
        xg_set_error(XIN_GPU_ERR_STATE, "fdct2_wxh_noalloc: call xin_gpu_init first");
        return XIN_GPU_ERR_STATE;
    }
    int dev = -1;
    if (xg_cuda_check(cudaGetDevice(&dev), "fdct2_wxh_noalloc: cudaGetDevice")) return XIN_GPU_ERR_CUDA;
    if (dev != g_device) {
        xg_set_error(XIN_GPU_ERR_STATE, "fdct2_wxh_noalloc: current device %d is not the library's device %d", dev, g_device);
        return XIN_GPU_ERR_STATE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    xg_coef *scratch = xg_noalloc_scratch(dev, st);
    if (!scratch) return xin_gpu_last_status();
    (void)cudaGetLastError();
    int n = (int)(width * height);
    k_fdct1d<<<(n + 255) / 256, 256, 0, st>>>(0, lw, input, (int)inputStride, scratch, (int)height, (int)height, shift1st);
    k_fdct1d<<<(n + 255) / 256, 256, 0, st>>>(0, lh, scratch, (int)height, output, (int)outputStride, (int)width, shift2nd);
    xg_count_launch(2);
    return xg_cuda_check(cudaGetLastError(), "fdct2_wxh_noalloc: launch");
}
