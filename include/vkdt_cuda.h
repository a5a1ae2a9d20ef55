/*
 * libvkdt_cuda: GB300 (sm_103a) CUDA backend for the raw development hot path
 * of vkdt:  denoise -> hilite -> demosaic -> colour -> filmcurv -> llap
 * over a 16-bit Bayer (rggb) or X-Trans mosaic.
 *
 * The library replaces, for those nodes, vkdt's Vulkan device layer (src/qvk)
 * and the modules' .comp shaders. Module names, parameters (the `params` files
 * of each module), connector formats (rggb:ui16 in, rgba:f16 out) and the .cfg
 * graph syntax are those of the reference. Every call returns an int that uses
 * the VkResult numbering the reference scheduler propagates with QVKR
 * (src/qvk/qvk.h): 0 success, negative errors, VK_INCOMPLETE (5) for a graph
 * the library cannot run. Nothing in the library aborts or exits.
 *
 * Threading: a graph is used by one thread at a time (src/pipe/graph.h:67-69);
 * different graphs may run concurrently on different streams.
 */
#ifndef VKDT_CUDA_H
#define VKDT_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VKDT_CUDA_API_VERSION 1

/* 8 character token packed into an int64, as src/pipe/token.h:15 */
typedef uint64_t dt_token_t;

/* return codes (VkResult numbering) */
#define VKDT_CUDA_SUCCESS                        0
#define VKDT_CUDA_NOT_READY                      1   /* VK_NOT_READY: job still running */
#define VKDT_CUDA_TIMEOUT                        2   /* VK_TIMEOUT: bounded wait ran out */
#define VKDT_CUDA_INCOMPLETE                     5   /* VK_INCOMPLETE: unconnected/unsupported graph */
#define VKDT_CUDA_ERROR_OUT_OF_HOST_MEMORY     (-1)
#define VKDT_CUDA_ERROR_OUT_OF_DEVICE_MEMORY   (-2)  /* allocation or admission failed */
#define VKDT_CUDA_ERROR_INITIALIZATION_FAILED  (-3)
#define VKDT_CUDA_ERROR_DEVICE_LOST            (-4)  /* device error or a device-side status word */
#define VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED  (-11)  /* bad sizes / parameters */
#define VKDT_CUDA_ERROR_UNKNOWN               (-13)

/* run flags: the s_graph_run_* bits of src/pipe/modules/api.h:25-37 */
#define VKDT_CUDA_RUN_ROI            (1u<<0)
#define VKDT_CUDA_RUN_CREATE_NODES   (1u<<1)
#define VKDT_CUDA_RUN_ALLOC          (1u<<2)
#define VKDT_CUDA_RUN_RECORD_CMD_BUF (1u<<3)
#define VKDT_CUDA_RUN_UPLOAD_SOURCE  (1u<<4)
#define VKDT_CUDA_RUN_DOWNLOAD_SINK  (1u<<5)
#define VKDT_CUDA_RUN_WAIT_DONE      (1u<<6)
#define VKDT_CUDA_RUN_ALL            (0xffffffffu)

/* image metadata the raw input module sets on its output
 * (dt_image_params_t, src/pipe/module.h:72-109; filled in
 * src/pipe/modules/i-raw/main.c:138-259) */
typedef struct vkdt_cuda_img_param_t
{
  float    black[4];           /* black level, raw DN */
  float    white[4];           /* white level, raw DN */
  float    whitebalance[4];    /* camera coefficients, normalised to green = 1 */
  uint32_t filters;            /* 0 rgb, 9 x-trans 6x6, else bayer rggb */
  uint32_t crop_aabb[4];       /* x0 y0 x1 y1 of the active area */
  float    cam_to_rec2020[9];  /* row major camera rgb -> linear rec2020 */
  float    noise_a;            /* noise profile, gaussian part (normalised units) */
  float    noise_b;            /* noise profile, poissonian part (normalised units) */
  uint32_t orientation;        /* exif orientation (crop's automatic rotation: 3, 6, 8) */
}
vkdt_cuda_img_param_t;

/* one node of the expanded graph, as the modules' create_nodes emit them
 * (dt_node_t, src/pipe/node.h:19-52): identity and dispatch size */
typedef struct vkdt_cuda_node_info_t
{
  dt_token_t name;     /* module directory, e.g. "hilite" */
  dt_token_t kernel;   /* kernel, e.g. "reduce" */
  uint32_t   wd, ht, dp;
  uint32_t   fused;    /* index of the CUDA kernel launch that computes this node */
}
vkdt_cuda_node_info_t;

typedef struct vkdt_cuda_graph_t vkdt_cuda_graph_t;

/* ---- device layer (replaces qvk_init/qvk_cleanup, src/cli/main.c:101,157) */

/* select and initialise a CUDA device. flags: reserved, pass 0 */
int  vkdt_cuda_init(int device_id, uint32_t flags);
void vkdt_cuda_cleanup(void);
/* 1 if the library runs node (name, kernel), e.g. ("llap", "assemble"):
 * the question dt_graph_create_shader_module asks (src/pipe/graph.c:303-343) */
int  vkdt_cuda_supports(dt_token_t name, dt_token_t kernel);

/* ---- graph (dt_graph_init/dt_graph_cleanup, src/pipe/graph.h:176-194) */

int  vkdt_cuda_graph_create(vkdt_cuda_graph_t **graph);
void vkdt_cuda_graph_destroy(vkdt_cuda_graph_t *graph);

/* read a .cfg graph (the text of e.g. bin/default-darkroom.i-raw) with the
 * line syntax of dt_graph_read_config_ascii (src/pipe/graph-io.c:232-282):
 * module:<name>:<inst>, connect:..., param:<name>:<inst>:<param>:<values>.
 * modules outside the path are recorded and reported by
 * vkdt_cuda_graph_unsupported(); the path must be connected i-raw:main ->
 * denoise -> hilite -> demosaic -> [crop] -> colour -> filmcurv -> llap. */
int  vkdt_cuda_graph_read_config(vkdt_cuda_graph_t *graph, const char *cfg, size_t len);
/* number of modules in the cfg the library does not run; names written as
 * tokens to `names` (up to max) */
int  vkdt_cuda_graph_unsupported(vkdt_cuda_graph_t *graph, dt_token_t *names, int max);

/* set/get a module parameter by name (dt_module_set_param_*, the values of a
 * `param:` cfg line). bytes must match count*4 of the params file entry. */
int  vkdt_cuda_graph_set_param(vkdt_cuda_graph_t *graph, dt_token_t module, dt_token_t inst,
    dt_token_t param, const void *value, size_t bytes);
int  vkdt_cuda_graph_get_param(vkdt_cuda_graph_t *graph, dt_token_t module, dt_token_t inst,
    dt_token_t param, void *value, size_t bytes);

/* source metadata: what i-raw's modify_roi_out provides (full size + img_param) */
int  vkdt_cuda_graph_set_input(vkdt_cuda_graph_t *graph, int wd, int ht, const vkdt_cuda_img_param_t *ip);
/* requested size of the output (the sink's roi). 0,0 = full size. a scale of
 * >= 3 (bayer) switches demosaic to its half-size + resample path */
int  vkdt_cuda_graph_set_output_size(vkdt_cuda_graph_t *graph, int wd, int ht);
/* llap pyramid depth override (0 = automatic as llap/main.c:44-89) */
int  vkdt_cuda_graph_set_llap_levels(vkdt_cuda_graph_t *graph, int levels);

/* run modify_roi/create_nodes for every module (no device work): the node
 * list becomes available through vkdt_cuda_graph_node*. */
int  vkdt_cuda_graph_create_nodes(vkdt_cuda_graph_t *graph);
/* run create_nodes for every module and allocate device memory
 * (dt_graph_run_modules + dt_graph_run_nodes_allocate, src/pipe/graph.c:747-806).
 * *device_bytes (may be 0) receives the bytes allocated. */
int  vkdt_cuda_graph_alloc(vkdt_cuda_graph_t *graph, uint64_t *device_bytes);
/* one node as the reference's scheduler holds it after the modules' create_nodes
 * and commit_params (dt_node_t, src/pipe/node.h:19-52), with its module's uniform
 * block (committed_param, or param where the module commits none, as
 * dt_graph_run_modules_upload_uniforms copies it, src/pipe/graph-run-modules.h:20-28) */
typedef struct vkdt_cuda_node_desc_t
{
  dt_token_t  name, kernel;    /* module directory and kernel (node.h: name, kernel) */
  int32_t     wd, ht, dp;      /* dispatch size (node.h: wd, ht, dp) */
  uint32_t    push_size;       /* node.h: push_constant_size (at most 256) */
  const void *push;            /* node.h: push_constant */
  uint32_t    uniform_size;    /* the module's uniform block size */
  const void *uniform;         /* the module's uniform block (std140 params_t) */
}
vkdt_cuda_node_desc_t;

/* the module layer's output in place of the library's own: replaces
 * dt_graph_run_nodes_record_cmd (src/pipe/graph.c:819) for the nodes of
 * denoise -> hilite -> demosaic -> colour -> filmcurv -> llap. in_wd x in_ht is
 * the i-raw output; nodes are the scheduler's nodes of those modules after
 * create_nodes and commit_params (any order; other modules' nodes absent).
 * The library reads the image metadata from the push constants (crop,
 * black/white, white balance, CFA, noise profile) and the module parameters
 * from the uniform blocks (colour's committed white balance multipliers,
 * exposure and camera matrix as they are), plans its fused launches, and
 * checks that they compute exactly these nodes: the same (name, kernel, wd,
 * ht, dp) multiset, apart from a shared:resample node at its input's size
 * (the identity the library folds away) and filmcurv's display node.
 * VKDT_CUDA_INCOMPLETE when the nodes are a chain the library does not run
 * (the caller keeps the reference's own device path for them). Then alloc and
 * run as after vkdt_cuda_graph_create_nodes. */
int  vkdt_cuda_graph_set_nodes(vkdt_cuda_graph_t *graph, int in_wd, int in_ht, const vkdt_cuda_node_desc_t *nodes,
    int count);

/* the node list create_nodes produced (for inspection and per-node timing) */
int  vkdt_cuda_graph_node_count(vkdt_cuda_graph_t *graph);
int  vkdt_cuda_graph_node(vkdt_cuda_graph_t *graph, int i, vkdt_cuda_node_info_t *info);
/* device bytes vkdt_cuda_graph_alloc takes for the graph as it is set up now
 * (runs create_nodes, allocates nothing); the allocated bytes once allocated */
int  vkdt_cuda_graph_plan_bytes(vkdt_cuda_graph_t *graph, uint64_t *device_bytes);
/* output size after alloc */
int  vkdt_cuda_graph_output_size(vkdt_cuda_graph_t *graph, int *wd, int *ht);

/* pinned host staging, valid until destroy (vkMapMemory of the staging
 * buffers, src/pipe/graph-run-nodes-upload.h:60-80, -download.h:17-26):
 * source = wd*ht uint16 mosaic, sink = out_wd*out_ht*4 IEEE half rgba */
void *vkdt_cuda_graph_map_source(vkdt_cuda_graph_t *graph, size_t *bytes);
void *vkdt_cuda_graph_map_sink(vkdt_cuda_graph_t *graph, size_t *bytes);
/* the resident device buffers behind source and sink */
int  vkdt_cuda_graph_device_buffers(vkdt_cuda_graph_t *graph, void **d_source, void **d_sink);

/* run the graph on `stream` (a cudaStream_t, 0 = the graph's own stream):
 * upload source (if flagged), all kernels, download sink (if flagged), wait
 * (if flagged). the dt_graph_run sequence of src/pipe/graph.c:719-936. */
int  vkdt_cuda_graph_run(vkdt_cuda_graph_t *graph, void *stream, uint32_t run_flags);
/* bounded wait for the last run: VKDT_CUDA_TIMEOUT after timeout_ms */
int  vkdt_cuda_graph_wait(vkdt_cuda_graph_t *graph, uint32_t timeout_ms);
/* develop from a device mosaic into a device rgba f16 buffer (resident data,
 * no host copies). both buffers as the graph's source/sink layouts. */
int  vkdt_cuda_graph_develop(vkdt_cuda_graph_t *graph, const void *d_mosaic, void *d_rgba, void *stream);

/* vkdt_cuda_graph_develop without any allocation, for small images.
 * No counterpart in the reference: there every buffer comes from the graph's
 * own Vulkan allocation (graph-run-nodes-allocate.h).
 *
 * For callers that must not allocate device memory at the moment they
 * develop (a display or video callback running beside busy streams, where
 * cudaMalloc/cudaFree may synchronise the device; an embedding that owns
 * every allocation). The intermediate buffers live in one fixed scratch array
 * of VKDT_CUDA_STATIC_SCRATCH_BYTES per device, reserved when the library's
 * CUDA module loads. The call makes no allocation of any kind.
 * - the graph has had vkdt_cuda_graph_set_input and vkdt_cuda_graph_create_nodes
 *   (after the last change of input, llap depth or output size) and is NOT
 *   allocated; debug stages, timing and the histogram need an allocated graph.
 * - d_mosaic and d_rgba are the caller's device buffers (source/sink layouts);
 *   stream is a cudaStream_t (0 = the legacy default stream).
 * - sizes whose intermediates exceed the scratch are rejected with
 *   VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED (about 17.5 bytes per pixel: up to
 *   about 1.9 megapixels, e.g. 1600x1200; 1920x1080 does not fit).
 * - nothing in the scratch has to start at zero: each call clears the part it
 *   uses on the stream before its kernels read it.
 * - all calls on one device share the one scratch: calls that overlap (from
 *   several threads, or on several streams before the earlier one finished)
 *   race and corrupt each other's results. Order them on one stream.
 * - the first call on each device looks up the scratch address
 *   (cudaGetSymbolAddress), which may load the CUDA module: make that first
 *   call before any stream capture begins. */
#define VKDT_CUDA_STATIC_SCRATCH_BYTES (32u << 20)
int  vkdt_cuda_graph_develop_static(vkdt_cuda_graph_t *graph, const void *d_mosaic, void *d_rgba, void *stream);

/* per-launch device times of the last run with timing enabled (the -d perf
 * output of src/pipe/graph.c:881-932): names are "module:kernel" tokens of
 * the fused launch. returns the count. */
int  vkdt_cuda_graph_set_timing(vkdt_cuda_graph_t *graph, int enable);
int  vkdt_cuda_graph_query_times(vkdt_cuda_graph_t *graph, float *ms, dt_token_t *names, dt_token_t *kernels, int max);

/* replay the launch sequence of a run as a captured CUDA graph (default 1):
 * captured on the first run, replayed while buffers and per-image values
 * stay the same, and updated in place (cudaGraphExecUpdate) after either
 * changes. 0 launches it eagerly every run. */
int  vkdt_cuda_graph_set_capture(vkdt_cuda_graph_t *graph, int enable);
/* the graph's own stream (a cudaStream_t), valid after alloc */
void *vkdt_cuda_graph_stream(vkdt_cuda_graph_t *graph);

/* ---- develop server: continuous batching of develop jobs on one device.
 * No counterpart in the reference, which runs one graph at a time; this is
 * the export daemon beside vkdt-cli. Jobs of any size are queued, admitted
 * while a slot is free and the device bytes of the graphs that run them stay
 * under the cap, and developed concurrently (one stream per graph). Every job
 * gets exactly the result it gets alone: same kernels, no shared state. */
typedef struct vkdt_cuda_server_t vkdt_cuda_server_t;

typedef struct vkdt_cuda_server_cfg_t
{
  const char *cfg;          /* graph .cfg text (module params), NULL = the darkroom path defaults */
  size_t      cfg_len;
  int         slots;        /* jobs in flight at once (streams), >= 1 */
  uint64_t    hbm_cap;      /* device bytes the server's graphs may hold, 0 = 90% of free memory */
  int         llap_levels;  /* llap pyramid depth, 0 = automatic */
}
vkdt_cuda_server_cfg_t;

typedef struct vkdt_cuda_job_t
{
  int         wd, ht;       /* mosaic size */
  vkdt_cuda_img_param_t ip; /* metadata of this image */
  int         out_wd, out_ht; /* requested output size, 0 = full size */
  const void *src;          /* uint16 mosaic, wd*ht, device or host (pinned for overlap) */
  void       *dst;          /* rgba f16 output at the output size, device or host */
  int         src_on_device, dst_on_device;
}
vkdt_cuda_job_t;

typedef struct vkdt_cuda_server_stats_t
{
  uint64_t completed, failed;
  double   mpix;            /* input megapixels of completed jobs */
  double   latency_p50_ms, latency_p99_ms;  /* submit -> done, completed jobs */
  uint64_t peak_device_bytes;
  int      graphs;          /* allocated graphs in the pool */
}
vkdt_cuda_server_stats_t;

int  vkdt_cuda_server_create(const vkdt_cuda_server_cfg_t *cfg, vkdt_cuda_server_t **server);
/* queue a job (the buffers must stay valid until it is done); *job_id names it */
int  vkdt_cuda_server_submit(vkdt_cuda_server_t *server, const vkdt_cuda_job_t *job, uint64_t *job_id);
/* bounded wait for one job: its status (0, or the error the develop returned),
 * VKDT_CUDA_TIMEOUT when timeout_ms passed first, VKDT_CUDA_NOT_READY for 0 ms */
int  vkdt_cuda_server_wait(vkdt_cuda_server_t *server, uint64_t job_id, uint32_t timeout_ms);
/* bounded wait for every queued and running job */
int  vkdt_cuda_server_drain(vkdt_cuda_server_t *server, uint32_t timeout_ms);
/* times of a finished job: queued (submit -> start) and latency (submit -> done), ms */
int  vkdt_cuda_server_job_times(vkdt_cuda_server_t *server, uint64_t job_id, double *queued_ms, double *latency_ms);
int  vkdt_cuda_server_stats(vkdt_cuda_server_t *server, vkdt_cuda_server_stats_t *stats);
/* forget the latency samples and counters (the pool of graphs stays) */
int  vkdt_cuda_server_reset_stats(vkdt_cuda_server_t *server);
void vkdt_cuda_server_destroy(vkdt_cuda_server_t *server);

/* 257 bin histogram the filmcurv module feeds to its display
 * (OpenDRT/hist.comp): bins 0..255 and the count in [256]. enable before run. */
int  vkdt_cuda_graph_set_hist(vkdt_cuda_graph_t *graph, int enable);
int  vkdt_cuda_graph_hist(vkdt_cuda_graph_t *graph, uint32_t *hist257);

/* standalone OpenDRT/hist.comp over a device rgba f16 image into a device u32[257]
 * (cleared by the call) */
int  vkdt_cuda_hist_rgba_f16(const void *d_rgba, int wd, int ht, uint32_t *d_hist257, void *stream);
/* hist/collect.comp:13-26 (the hist module's collect node, hist/main.c:26-41):
 * the rgb waveform of a device rgba f16 image into a device u32 image of
 * out_wd x out_ht (the module asks 1000 x 600, hist/main.c:9-11), cleared
 * first as the node's s_conn_clear output is. Column int(out_wd/wd * x), row
 * (1 - value) * out_ht + 0.5 (negative and NaN count in row 0, values past the
 * last row in the last); red adds 1, green 1024, blue 1048576. Exact integer
 * counts; does not wait for its stream. */
int  vkdt_cuda_waveform_rgba_f16(const void *d_rgba, int wd, int ht, uint32_t *d_out, int out_wd, int out_ht,
    void *stream);

/* lens/main.comp:22-57 (the lens module, declared in bin/default-darkroom.i-raw; no host
 * code: its params file is the uniform block): a device rgba f16 image of wd x ht resampled
 * into a device rgba f16 image of out_wd x out_ht (the module's output has the input's size)
 * through the double sphere camera model. params in the params file's order: centre x, y,
 * scale x, y, squish0, squish1, ca red, ca blue (lens/params; defaults 0 0 1 1 0 0 1 1).
 * Catmull-Rom sampling (shared.glsl sample_catmull_rom), alpha 1. 8-byte aligned buffers.
 * Asynchronous on `stream`. */
int  vkdt_cuda_lens_rgba_f16(const void *d_in, int wd, int ht, void *d_out, int out_wd, int out_ht,
                             const float params[8], void *stream);

/* Ingestion of packed raw video (replaces the host unpack of i-mlv/video_mlv.c:254-274,
 * called from read_source at i-mlv/main.c:204-211 through read_frame at main.c:76-85):
 * d_packed holds an uncompressed magic lantern frame of `bytes` bytes (16-bit aligned) with
 * bits_per_pixel 10, 12, 14 or 16; d_mosaic (wd*ht u16, e.g. a graph's device source from
 * vkdt_cuda_graph_device_buffers) receives the samples. Asynchronous on `stream`.
 * VK_ERROR_FORMAT_NOT_SUPPORTED for another bit depth, an unaligned pointer or a frame
 * shorter than wd*ht*bits_per_pixel/8 bytes. */
int  vkdt_cuda_unpack_mlv(const void *d_packed, size_t bytes, int bits_per_pixel, int wd, int ht, void *d_mosaic,
                          void *stream);

/* Ingestion of motioncam raw video (replaces the i-mcraw nodes prefix and decode,
 * i-mcraw/main.cc:366-408 create_nodes, i-mcraw/prefix.comp, i-mcraw/decode.comp): the
 * frame's source buffers as i-mcraw's read_source fills them (main.cc:411-446) on the
 * device: d_bitcnt (one 4-bit count per block of 64 samples, two per byte, low nibble
 * first), d_refval (u16 per block), d_data (data_bytes of block data). rwd x ht is the
 * encoded size (rwd a multiple of 64, ht of 4); d_mosaic receives the wd x hgt u16 mosaic
 * offset by (ox, oy) (modify_roi_out at main.cc:330-360), each sample as the reference's
 * R16_UNORM store of (reference + delta) / 65536 leaves it. d_scratch: at least
 * vkdt_cuda_mcraw_scratch_bytes(rwd, ht) bytes, 8-byte aligned. Asynchronous on `stream`. */
size_t vkdt_cuda_mcraw_scratch_bytes(int rwd, int ht);
int  vkdt_cuda_mcraw_decode(const void *d_bitcnt, const void *d_refval, const void *d_data, size_t data_bytes,
                            int rwd, int ht, int ox, int oy, int wd, int hgt, void *d_mosaic, void *d_scratch,
                            void *stream);

/* Output encode after the path (the thumbnail graph's tail, bin/default.i-raw:9-10,16-17).
 * vkdt_cuda_colenc replaces colenc/main.comp (colenc/main.c create_nodes): rec2020 linear rgba f16
 * to the output primaries (the colenc `prim` param: 1 rec709, 3 adobergb, 4 p3d65, 5 xyz, 6 ap0,
 * 7 ap1, 10 redwg, others unchanged) and transfer curve (`trc`: 0 linear, 1 709, 2 sRGB, 3 PQ,
 * 4 DCI, 5 HLG, 6 gamma 2.2), written as rgba f16 to d_out_f16 and/or as the rgba u8 an 8-bit sink
 * reads (R8G8B8A8_UNORM stores, alpha 255) to d_out_u8 (either may be null).
 * vkdt_cuda_bc1_encode replaces o-bc1's host encoder (o-bc1/main.c:21-47, stb_dxt.h): the BC1
 * blocks (8 bytes each, row major) of the whole 4x4 blocks of an rgba u8 image; d_rgba_u8 4-byte
 * aligned. Both asynchronous on `stream`. */
int  vkdt_cuda_colenc(const void *d_rgba_f16, int wd, int ht, int primaries, int trc, void *d_out_f16, void *d_out_u8,
                      void *stream);
int  vkdt_cuda_bc1_encode(const void *d_rgba_u8, int wd, int ht, void *d_blocks, void *stream);

/* ---- noise statistics and the noise profile fit (rawhist and nprof modules)
 *
 * rawhist/collect.comp:22-66 over a device mosaic (uint16, row pitch = wd):
 * per CFA block the green cross mean and second moment of the black/white
 * normalised values, binned by bins*log2(mean+1). h_out (host, 3*bins
 * doubles) receives per bin the block count, the sum of means and the sum of
 * second moments (exact: 64-bit fixed point sums, one FP64 combine). black
 * and white are those of the metadata's channel 1, as rawhist/main.c:17-28
 * commits them. d_scratch: device memory of vkdt_cuda_rawhist_scratch_bytes().
 * The call waits for its stream. bins <= 1024 (the reference uses 1000). */
size_t vkdt_cuda_rawhist_scratch_bytes(void);
int  vkdt_cuda_rawhist(const void *d_mosaic, int wd, int ht, const vkdt_cuda_img_param_t *ip, int bins,
    void *d_scratch, double *h_out, void *stream);
/* nprof/main.c:82-198 on such a histogram: outlier rejecting pair fits of
 * sigma^2 = a + b x between bins, then the count weighted regression over
 * the accepted bins; a, b in the normalised units of vkdt_cuda_img_param_t.
 * Host code, no device work. */
int  vkdt_cuda_nprof_fit(const double *hist, int bins, float *a, float *b);

/* debug: copy an intermediate image of the last run to host floats.
 * stage 0 denoise output (1 ch), 1 hilite output (1 ch), both at the crop size;
 * 2 filmcurv output and 4 colour output (4 ch each) at the output size; 3
 * demosaic output (4 ch) at the demosaic's size (the output size unless crop
 * follows it); 11 crop output (4 ch, the output size; only when crop moves
 * pixels); with the wavelet denoise, its half size nodes (4 ch, W/block x
 * H/block): 5 half, 6 downcov, 7..9 down levels 1..3 (swizzled as
 * denoise/down.comp:102-104 stores them), 10 assemble. These are the images the reference's `-d perf` graph
 * would hold on those nodes' output connectors (graph.c:881-932).
 * requires vkdt_cuda_graph_set_debug(graph, 1) before alloc (stage 2 does not).
 * vkdt_cuda_graph_debug_stage_size gives a stage's width, height and channels. */
int  vkdt_cuda_graph_set_debug(vkdt_cuda_graph_t *graph, int enable);
int  vkdt_cuda_graph_debug_stage(vkdt_cuda_graph_t *graph, int stage, float *out, size_t count);
int  vkdt_cuda_graph_debug_stage_size(vkdt_cuda_graph_t *graph, int stage, int *wd, int *ht, int *channels);
/* debug: the discrete decisions the last run took, one element per texel of
 * a wd x ht grid (written to *wd, *ht; out may be null to ask for the size).
 * kind 0: demosaic/gauss.comp per entry (W/block x H/block), u8: bit 0 the
 *         structure tensor taken was Sw (det(Sw) < det(Sb), gauss.comp:65,117),
 *         bits 1-2 the snapped direction 0 (1,0), 1 (0,1), 2 none (x-trans
 *         isotropic; gauss.comp:72-73, 121-123);
 * kind 1: denoise/cov.glsl response() per half size texel, u32: bits 0-24
 *         tap (i+2)+5(j+2) skipped as a hot pixel (cov.glsl:130), bit 25 Sw
 *         taken (cov.glsl:84);
 * kind 2: denoise/assemble.comp per half size texel, u8: bit l set where the
 *         coarse threshold switch |d_l| > 10 fired (assemble.comp:144-153).
 * No reference counterpart: these let a test show that every result that
 * differs from the reference's arithmetic does so where a branch of the
 * reference was a near tie. requires debug stages enabled before alloc. */
int  vkdt_cuda_graph_debug_decisions(vkdt_cuda_graph_t *graph, int kind, void *out, size_t bytes, int *wd, int *ht);

/* ---- synthetic raw scenes (the seeded mosaics the benchmarks are quoted on) */

typedef struct vkdt_cuda_scene_t
{
  int32_t  wd, ht;
  uint32_t seed, image_id;
  uint32_t filters;           /* cfa of the mosaic (bayer rggb or 9) */
  float    black, white;      /* DN */
  float    noise_a, noise_b;  /* DN: variance = a + b * signal */
  float    wb[3];             /* camera rgb = scene / wb */
  float    pan_x, pan_y;      /* scene offset in pixels (video panning) */
}
vkdt_cuda_scene_t;

/* fill a device (or host) u16 mosaic with the seeded scene */
int  vkdt_cuda_scene_generate(const vkdt_cuda_scene_t *scene, void *d_mosaic, void *stream);
int  vkdt_cuda_scene_generate_host(const vkdt_cuda_scene_t *scene, uint16_t *mosaic);

/* last error message of this thread (static storage) */
const char *vkdt_cuda_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
