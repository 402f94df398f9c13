/*
 * TEST INFRASTRUCTURE ONLY — the CPU oracle for the STFT hot path.
 *
 * Nothing in the product (occastft_gb300/, include/) links or calls this code.
 * It is used by tests/ (parity checks), __graft_entry__.smoke() (one check of
 * the CUDA path) and bench.py (the timed CPU baseline / reference arm).
 *
 * Two oracles live here:
 *   orc_serial_pipeline — a restatement, operation for operation, of the
 *       reference's Serial/OpenMP runner pipeline (float32, cosf/sinf per
 *       butterfly, including the reference's quirks).  It is pinned
 *       bit-for-bit against the reference's own code compiled from source
 *       (oracle/build_ref.sh) and against the committed golden vectors.
 *   orc_fp64_stft — the same framing and window coefficients, with DC removal
 *       and the FFT done in double precision: the accuracy reference.
 */
#ifndef OCS_STFT_ORACLE_H
#define OCS_STFT_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* window kinds, in the precedence order of the reference's option chain */
enum {
    ORC_WIN_NONE = 0,
    ORC_WIN_HANNING = 1,
    ORC_WIN_HAMMING = 2,
    ORC_WIN_BLACKMAN = 3,
    ORC_WIN_NUTTALL = 4,
    ORC_WIN_BLACKMAN_NUTTALL = 5,
    ORC_WIN_BLACKMAN_HARRIS = 6,
    ORC_WIN_FLATTOP = 7,
    ORC_WIN_GAUSSIAN = 8
};

typedef struct {
    int window;          /* ORC_WIN_* */
    float sigma;         /* gaussian sigma as the reference parses it */
    int remove_dc;       /* --remove_dc */
    int half_complex;    /* --half_complex_return */
    int dense;           /* --layout=dense (extension: N/2+1 bins per frame) */
    int serial_power;    /* --serial_power (extension: the Serial runner's sqrt(2)|Re X|) */
} orc_options;

typedef struct {
    uint32_t qt;         /* toQuot frame count */
    uint32_t hop;        /* OMove */
    uint32_t ofull;      /* OFullSize = qt * N */
    uint32_t ohalf;      /* OHalfSize = OFullSize / 2 */
    uint32_t n_window;   /* N = 1 << exp */
} orc_geometry;

/* 0 on success, -1 when the reference would not run (exp < 6, overlap >= 1 ...) */
int orc_geometry_get(uint32_t n, int exp, float overlap, orc_geometry* g);
/* 0 = OK; otherwise writes the reference's status string into err */
int orc_parse_options(const char* options, orc_options* o, char* err, size_t errcap);
float orc_window_value(int kind, int index, int n_window, float sigma);
/* out must hold g.ofull floats; returns 0 or the parse error code */
int orc_serial_pipeline(const float* in, uint32_t n, int exp, float overlap,
                        const char* options, float* out, int fix_p4, int nthreads);
uint64_t orc_output_floats(const orc_geometry* g, const orc_options* o);
int orc_fp64_stft(const float* in, uint32_t n, int exp, float overlap,
                  const char* options, double* out, uint64_t out_cap, int nthreads);
/* 1: evaluate window coefficients per sample and twiddles per butterfly, as
 * the reference does (same values; used to time the CPU baseline at the
 * reference's cost); 0: per-call tables (default) */
void orc_set_reference_cost(int on);
/* per-stage restatements (float32) */
void orc_overlap(const float* in, uint32_t ofull, uint32_t n, uint32_t exp, uint32_t hop, float* real);
void orc_apply_window(int kind, float* data, uint32_t ofull, uint32_t n_window, float sigma, int nthreads);
void orc_remove_dc(float* data, uint32_t ofull, uint32_t n_window, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
