// window.cu -- mate-rescue windows fetched on the device from a reference held
// in HBM (matesw_collect and bns_fetch_seq, crates/bwa-mem/src/pe.rs:232-270 and
// :596-679; the 2-bit unpack of crates/bwa-index/src/fmindex.rs:162-185; the
// contig search of crates/bwa-index/src/bntseq.rs:337-365).
//
// A request names an anchor (its rb and contig), an orientation and the insert
// window; the mate read comes along.  One thread per request plans the window:
// the orientation's interval around the anchor, clamped to [0, 2*l_pac) and to
// the contig holding its midpoint (mirrored onto the reverse half), accepted when
// that contig is the anchor's and at least min_seed_len bases remain.  A scan lays
// the mates and windows out in HBM; one warp per request writes the mate
// (reverse-complemented for the reverse orientations) and unpacks the window
// from the packed reference, lanes over bases.  The rescue kernels then run on
// the accepted windows; the host receives each window and its alignment.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>

#include <cub/device/device_scan.cuh>

#include "kernels.h"
#include "runtime.h"

namespace bwacuda {

namespace {

struct WinReqDev {
    uint64_t mate_off;  // byte offset of the mate in the staged mates
    int64_t anchor_rb;
    int32_t l_ms, orient, anchor_rid, low, high, pad;
};
static_assert(sizeof(WinReqDev) == 40, "request layout");

struct WinInfo {
    int64_t rb, re;
    int32_t rid, valid;
};

struct RefView {
    const uint8_t *pac;
    const int64_t *off;
    const int32_t *len;
    int64_t l_pac;
    int32_t n;
};

// bns_pos2rid as the reference writes it: the last probe of its binary search.
__device__ int pos2rid(const RefView &R, int64_t pos_f)
{
    if (pos_f >= R.l_pac) return -1;
    int left = 0, mid = 0, right = R.n;
    while (left < right) {
        mid = (left + right) >> 1;
        if (pos_f >= R.off[mid]) {
            if (mid == R.n - 1) break;
            if (pos_f < R.off[mid + 1]) break;
            left = mid + 1;
        } else {
            right = mid;
        }
    }
    return mid;
}

// Base at 2L-space position p: forward unpack below l_pac, complement of the mirror above.
__device__ __forceinline__ uint8_t ref_base(const RefView &R, int64_t p)
{
    const bool rc = p >= R.l_pac;
    const int64_t f = rc ? 2 * R.l_pac - 1 - p : p;
    const uint32_t b = (R.pac[f >> 2] >> ((3 - (int)(f & 3)) << 1)) & 3u;
    return (uint8_t)(rc ? 3u - b : b);
}

// A request as the kernels see it: staged (WinReqDev, mates in a staging buffer)
// or the caller's own bwacuda_window_req read in place (mates at their pointers).
struct ReqView {
    const WinReqDev *staged;
    const bwacuda_window_req *direct;
    const uint8_t *mates;  // staged mates
    __device__ __forceinline__ WinReqDev get(uint32_t k, const uint8_t **mate) const
    {
        if (staged) {
            const WinReqDev q = staged[k];
            *mate = mates + q.mate_off;
            return q;
        }
        const bwacuda_window_req r = direct[k];
        WinReqDev q;
        q.mate_off = 0;
        q.anchor_rb = r.anchor_rb;
        q.l_ms = r.l_ms;
        q.orient = r.orient;
        q.anchor_rid = r.anchor_rid;
        q.low = r.low;
        q.high = r.high;
        q.pad = 0;
        *mate = r.mate;
        return q;
    }
};

__global__ void win_plan_kernel(const ReqView V, uint32_t n, const RefView R, int min_seed_len,
                                WinInfo *__restrict__ info, uint64_t *__restrict__ sizes,
                                unsigned long long *__restrict__ cells)
{
    unsigned long long my_cells = 0;  // qlen x tlen of the accepted windows (the statistics)
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint8_t *unused;
        const WinReqDev q = V.get(k, &unused);
        const int r = q.orient;
        const bool is_rev = (r >> 1) != (r & 1);
        const bool is_larger = (r >> 1) == 0;
        const int64_t lo = q.low, hi = q.high, l_ms = q.l_ms;
        int64_t rb, re;
        if (!is_rev) {
            rb = is_larger ? q.anchor_rb + lo : q.anchor_rb - hi;
            re = (is_larger ? q.anchor_rb + hi : q.anchor_rb - lo) + l_ms;
        } else {
            rb = (is_larger ? q.anchor_rb + lo : q.anchor_rb - hi) - l_ms;
            re = is_larger ? q.anchor_rb + hi : q.anchor_rb - lo;
        }
        rb = rb > 0 ? rb : 0;
        re = re < (R.l_pac << 1) ? re : (R.l_pac << 1);
        WinInfo w{rb, re, -1, 0};
        if (rb < re) {
            // bns_fetch_seq(rb, (rb + re) >> 1, re): clamp to the midpoint's contig
            const int64_t mid = (rb + re) >> 1;
            const bool mrev = mid >= R.l_pac;
            const int64_t mid_f = mrev ? (R.l_pac << 1) - 1 - mid : mid;
            const int rid = pos2rid(R, mid_f);
            int64_t far_beg = 0, far_end = R.l_pac << 1;
            if (rid >= 0) {
                far_beg = R.off[rid];
                far_end = R.off[rid] + (int64_t)R.len[rid];
                if (mrev) {
                    const int64_t fb = far_beg;
                    far_beg = (R.l_pac << 1) - far_end;
                    far_end = (R.l_pac << 1) - fb;
                }
            }
            w.rb = rb > far_beg ? rb : far_beg;
            w.re = re < far_end ? re : far_end;
            w.rid = rid;
            w.valid = (rid == q.anchor_rid && w.re - w.rb >= (int64_t)min_seed_len) ? 1 : 0;
        }
        info[k] = w;
        sizes[k] = (uint64_t)q.l_ms + (w.valid ? (uint64_t)(w.re - w.rb) : 0u);
        if (w.valid) my_cells += (unsigned long long)q.l_ms * (unsigned long long)(w.re - w.rb);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) my_cells += __shfl_xor_sync(0xffffffffu, my_cells, o);
    if ((threadIdx.x & 31u) == 0 && my_cells) atomicAdd(cells, my_cells);
}

// One warp per request: the mate (reverse-complemented for the reverse orientations)
// and the window bases, then the rescue descriptor.
__global__ void win_fill_kernel(const ReqView V, uint32_t n, const RefView R, const WinInfo *__restrict__ info,
                                const uint64_t *__restrict__ offs, uint8_t *__restrict__ seq,
                                bwacuda_dev_rescue_job *__restrict__ jobs)
{
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n; k += (gridDim.x * blockDim.x) >> 5) {
        const uint8_t *ms;
        const WinReqDev q = V.get(k, &ms);
        const WinInfo w = info[k];
        const int r = q.orient;
        const bool is_rev = (r >> 1) != (r & 1);
        uint8_t *dq = seq + offs[k];
        const int lq = w.valid ? q.l_ms : 0;
        for (int x = (int)lane; x < lq; x += 32) {
            uint8_t b;
            if (is_rev) {
                const uint8_t c = ms[q.l_ms - 1 - x];
                b = c < 4 ? (uint8_t)(3 - c) : (uint8_t)4;
            } else {
                b = ms[x];
            }
            dq[x] = b;
        }
        const int64_t L = w.valid ? w.re - w.rb : 0;
        uint8_t *dt = dq + lq;
        for (int64_t x = lane; x < L; x += 32) dt[x] = ref_base(R, w.rb + x);
        if (lane == 0) {
            bwacuda_dev_rescue_job J;
            J.q_off = offs[k];
            J.t_off = offs[k] + (uint64_t)lq;
            J.qlen = lq;
            J.tlen = (int32_t)L;
            J.minsc = 0;
            J.endsc = 0;
            jobs[k] = J;
        }
    }
}

// The caller's result records, written in place (window and alignment per request).
// Records into a device buffer (one thread per request); win_copy_kernel then moves them to
// the caller's array word by word, so consecutive threads store consecutive host words.
__global__ void win_store_kernel(const WinInfo *__restrict__ info, const bwacuda_rescue_result *__restrict__ aln,
                                 uint32_t n, bwacuda_window_result *__restrict__ out)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const WinInfo w = info[k];
        bwacuda_window_result o;
        o.rb = w.rb;
        o.re = w.re;
        o.rid = w.rid;
        o.valid = w.valid;
        o.aln = aln[k];
        out[k] = o;
    }
}

__global__ void win_copy_kernel(const uint32_t *__restrict__ src, size_t words, uint32_t *__restrict__ dst)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

}  // namespace

struct RefState {
    DevBuf pac, off, len;
    int64_t l_pac = 0;
    int32_t n = 0;
    // per-call buffers
    DevBuf reqs, mates, info, sizes, offs, tmp, seq, jobs, res, outd;
    HostBuf h_reqs, h_tot;
};

void ref_release(bwacuda_ctx *c)
{
    if (!c->ref) return;
    RefState &S = *c->ref;
    S.pac.release(); S.off.release(); S.len.release();
    S.reqs.release(); S.mates.release(); S.info.release(); S.sizes.release(); S.offs.release(); S.tmp.release();
    S.seq.release(); S.jobs.release(); S.res.release(); S.outd.release(); S.h_reqs.release(); S.h_tot.release();
    delete c->ref;
    c->ref = nullptr;
}

}  // namespace bwacuda

using namespace bwacuda;

extern "C" int bwacuda_ref_set(bwacuda_ctx *c, const uint8_t *pac, int64_t l_pac, const int64_t *contig_offset,
                               const int32_t *contig_len, int32_t n_contigs)
{
    if (!c || !pac || l_pac <= 0 || !contig_offset || !contig_len || n_contigs <= 0) return BWACUDA_EINVAL;
    // offsets ascending from 0, every contig inside the forward reference
    for (int32_t i = 0; i < n_contigs; ++i) {
        if (contig_len[i] < 0 || contig_offset[i] < 0 || contig_offset[i] + contig_len[i] > l_pac) return BWACUDA_EINVAL;
        if (i == 0 ? contig_offset[i] != 0 : contig_offset[i] <= contig_offset[i - 1]) return BWACUDA_EINVAL;
    }
    std::lock_guard<std::mutex> g(c->mu);
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    if (!c->ref) {
        c->ref = new (std::nothrow) RefState();
        if (!c->ref) return BWACUDA_ENOMEM;
    }
    RefState &S = *c->ref;
    const size_t pac_bytes = (size_t)((l_pac + 3) >> 2);
    cudaError_t e;
    if ((e = S.pac.ensure(pac_bytes + 16)) != cudaSuccess) return cuda_status(e);
    if ((e = S.off.ensure((size_t)n_contigs * 8)) != cudaSuccess) return cuda_status(e);
    if ((e = S.len.ensure((size_t)n_contigs * 4)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaMemcpy(S.pac.p, pac, pac_bytes, cudaMemcpyHostToDevice)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaMemcpy(S.off.p, contig_offset, (size_t)n_contigs * 8, cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_status(e);
    if ((e = cudaMemcpy(S.len.p, contig_len, (size_t)n_contigs * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_status(e);
    S.l_pac = l_pac;
    S.n = n_contigs;
    c->stats.h2d_bytes += pac_bytes + (size_t)n_contigs * 12;
    return BWACUDA_OK;
}

extern "C" int bwacuda_mate_rescue_windows(bwacuda_ctx *c, const bwacuda_window_req *reqs, size_t n, int m,
                                           const int8_t *mat, int o_del, int e_del, int o_ins, int e_ins, int minsc,
                                           int max_sc, int min_seed_len, bwacuda_window_result *out)
{
    if (!c) return BWACUDA_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    int rc = validate_scoring(m, mat, o_del, e_del, o_ins, e_ins);
    if (rc) return rc;
    if (max_sc < 1 || (n && (!reqs || !out))) return BWACUDA_EINVAL;
    if (n == 0) return BWACUDA_OK;
    if (!c->ref || c->ref->l_pac <= 0) return BWACUDA_EINVAL;  // bwacuda_ref_set first
    if (n > ((size_t)1 << 30)) return BWACUDA_EUNSUPPORTED;
    uint64_t mate_bytes = 0;
    for (size_t k = 0; k < n; ++k) {
        const bwacuda_window_req &q = reqs[k];
        if (q.l_ms < 0 || (q.l_ms && !q.mate) || q.orient < 0 || q.orient > 3) return BWACUDA_EINVAL;
        mate_bytes += (uint64_t)q.l_ms;
    }
    if (cudaSetDevice(c->device) != cudaSuccess) return BWACUDA_ECUDA;
    RefState &S = *c->ref;
    cudaStream_t s = c->stream;
    cudaError_t e;
    // where the device reads pageable host memory the kernels read the caller's requests and
    // mates in place; otherwise they are staged through pinned memory
    const bool direct = c->pageable_access && c->host_gather != BWACUDA_GATHER_HOST;
    const size_t rq_bytes = n * sizeof(WinReqDev);
    if (!direct) {
        if ((e = S.h_reqs.ensure(rq_bytes + mate_bytes + 16)) != cudaSuccess) return cuda_status(e);
        WinReqDev *hr = static_cast<WinReqDev *>(S.h_reqs.p);
        uint8_t *hm = reinterpret_cast<uint8_t *>(hr + n);
        uint64_t mo = 0;
        for (size_t k = 0; k < n; ++k) {
            const bwacuda_window_req &q = reqs[k];
            WinReqDev d;
            d.mate_off = mo;
            d.anchor_rb = q.anchor_rb;
            d.l_ms = q.l_ms;
            d.orient = q.orient;
            d.anchor_rid = q.anchor_rid;
            d.low = q.low;
            d.high = q.high;
            d.pad = 0;
            hr[k] = d;
            if (q.l_ms) memcpy(hm + mo, q.mate, (size_t)q.l_ms);
            mo += (uint64_t)q.l_ms;
        }
    }
    size_t scan_bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (const uint64_t *)nullptr, (uint64_t *)nullptr, (int)n + 1);
    if (!direct && (e = S.reqs.ensure(rq_bytes + mate_bytes + 16)) != cudaSuccess) return cuda_status(e);
    if ((e = S.info.ensure(n * sizeof(WinInfo))) != cudaSuccess) return cuda_status(e);
    if ((e = S.sizes.ensure((n + 2) * 8)) != cudaSuccess) return cuda_status(e);
    if ((e = S.offs.ensure((n + 1) * 8)) != cudaSuccess) return cuda_status(e);
    if ((e = S.tmp.ensure(scan_bytes + 16)) != cudaSuccess) return cuda_status(e);
    if ((e = S.h_tot.ensure(64)) != cudaSuccess) return cuda_status(e);
    if ((e = S.jobs.ensure(n * sizeof(bwacuda_dev_rescue_job))) != cudaSuccess) return cuda_status(e);
    if ((e = S.res.ensure(n * sizeof(bwacuda_rescue_result))) != cudaSuccess) return cuda_status(e);
    ReqView V{nullptr, nullptr, nullptr};
    if (direct) {
        V.direct = reqs;
    } else {
        if ((e = cudaMemcpyAsync(S.reqs.p, S.h_reqs.p, rq_bytes + mate_bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return cuda_status(e);
        c->stats.h2d_bytes += rq_bytes + mate_bytes;
        V.staged = static_cast<const WinReqDev *>(S.reqs.p);
        V.mates = reinterpret_cast<const uint8_t *>(V.staged + n);
    }
    WinInfo *info = static_cast<WinInfo *>(S.info.p);
    uint64_t *sizes = static_cast<uint64_t *>(S.sizes.p), *offs = static_cast<uint64_t *>(S.offs.p);
    RefView R{static_cast<const uint8_t *>(S.pac.p), static_cast<const int64_t *>(S.off.p),
              static_cast<const int32_t *>(S.len.p), S.l_pac, S.n};
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || nsm < 1) nsm = 1;
    if ((e = cudaMemsetAsync(sizes + n, 0, 8, s)) != cudaSuccess) return cuda_status(e);
    // the accepted windows' cells, counted by the plan kernel (sizes[n + 1], after the scan's input)
    unsigned long long *d_cells = reinterpret_cast<unsigned long long *>(sizes + n + 1);
    if ((e = cudaMemsetAsync(d_cells, 0, 8, s)) != cudaSuccess) return cuda_status(e);
    uint32_t grid = (uint32_t)std::min<size_t>((n + 255) / 256, (size_t)nsm * 8);
    win_plan_kernel<<<grid, 256, 0, s>>>(V, (uint32_t)n, R, min_seed_len, info, sizes, d_cells);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
    if ((e = cub::DeviceScan::ExclusiveSum(S.tmp.p, scan_bytes, sizes, offs, (int)n + 1, s)) != cudaSuccess)
        return cuda_status(e);
    if ((e = cudaMemcpyAsync(S.h_tot.p, offs + n, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_status(e);
    if ((e = cudaMemcpyAsync(static_cast<uint64_t *>(S.h_tot.p) + 1, d_cells, 8, cudaMemcpyDeviceToHost, s)) !=
        cudaSuccess)
        return cuda_status(e);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status(e);
    const uint64_t total = *static_cast<const uint64_t *>(S.h_tot.p);
    const uint64_t cells = static_cast<const uint64_t *>(S.h_tot.p)[1];
    if ((e = S.seq.ensure(total + 16)) != cudaSuccess) return cuda_status(e);
    grid = (uint32_t)std::min<size_t>((n * 32 + 255) / 256, (size_t)nsm * 16);
    win_fill_kernel<<<grid, 256, 0, s>>>(V, (uint32_t)n, R, info, offs, static_cast<uint8_t *>(S.seq.p),
                                         static_cast<bwacuda_dev_rescue_job *>(S.jobs.p));
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
    c->stats.kernel_launches += 4;
    bwacuda_scoring sc;
    sc.m = m;
    memset(sc.mat, 0, sizeof(sc.mat));
    memcpy(sc.mat, mat, (size_t)m * m);
    sc.o_del = o_del; sc.e_del = e_del; sc.o_ins = o_ins; sc.e_ins = e_ins;
    rc = ksw_align2_device_locked(c, static_cast<const uint8_t *>(S.seq.p),
                                  static_cast<const bwacuda_dev_rescue_job *>(S.jobs.p), n, &sc, minsc, max_sc, 0, 0,
                                  static_cast<bwacuda_rescue_result *>(S.res.p), s);
    if (rc) return rc;
    if (direct) {
        // the records, assembled in HBM, then word by word straight into the caller's array
        if ((e = S.outd.ensure(n * sizeof(bwacuda_window_result))) != cudaSuccess) return cuda_status(e);
        grid = (uint32_t)std::min<size_t>((n + 255) / 256, (size_t)nsm * 8);
        win_store_kernel<<<grid, 256, 0, s>>>(info, static_cast<const bwacuda_rescue_result *>(S.res.p), (uint32_t)n,
                                              static_cast<bwacuda_window_result *>(S.outd.p));
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
        const size_t words = n * (sizeof(bwacuda_window_result) / 4);
        grid = (uint32_t)std::min<size_t>((words + 255) / 256, (size_t)nsm * 8);
        win_copy_kernel<<<grid, 256, 0, s>>>(static_cast<const uint32_t *>(S.outd.p), words,
                                             reinterpret_cast<uint32_t *>(out));
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
        uint64_t dummy = 0;
        if ((rc = collect_device_status(c, s, &dummy)) != BWACUDA_OK) return rc;  // synchronises
    } else {
        // windows and alignments back through the staging buffer, then into the caller's records
        if ((e = S.h_reqs.ensure(n * (sizeof(WinInfo) + sizeof(bwacuda_rescue_result)) + 16)) != cudaSuccess)
            return cuda_status(e);
        WinInfo *hi = static_cast<WinInfo *>(S.h_reqs.p);
        bwacuda_rescue_result *ha = reinterpret_cast<bwacuda_rescue_result *>(hi + n);
        if ((e = cudaMemcpyAsync(hi, info, n * sizeof(WinInfo), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return cuda_status(e);
        if ((e = cudaMemcpyAsync(ha, S.res.p, n * sizeof(bwacuda_rescue_result), cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess)
            return cuda_status(e);
        uint64_t dummy = 0;
        if ((rc = collect_device_status(c, s, &dummy)) != BWACUDA_OK) return rc;  // synchronises
        for (size_t k = 0; k < n; ++k) {
            bwacuda_window_result &o = out[k];
            o.rb = hi[k].rb;
            o.re = hi[k].re;
            o.rid = hi[k].rid;
            o.valid = hi[k].valid;
            o.aln = ha[k];
        }
    }
    c->stats.d2h_bytes += n * (sizeof(WinInfo) + sizeof(bwacuda_rescue_result));
    c->stats.rescue_cells += cells;
    return BWACUDA_OK;
}
