// tddump.cu -- time-domain field dumps of the GB300 engine: the counterpart of ProcessFieldsTD
// (Common/processfields_td.cpp:50-91) writing VTK XML rectilinear-grid files like
// VTK_File_Writer::WriteXML (tools/vtk_file_writer.cpp:312-371).
//
// Data path, with the simulation never waiting for the disk:
//   1. the step-end kernel writes each sample (the dump box's E or H, interpolated as the dump
//      mode says) into a ring of device slots;
//   2. after each chunk of graph replays the host enqueues, on the engine stream, one
//      cudaMemcpyAsync per new sample into a pinned host buffer plus an event. Stream order keeps
//      a slot from being overwritten before its copy ran; a chunk never produces more samples
//      than the ring holds;
//   3. a writer thread per engine waits for each event, transposes the sample to VTK point
//      order (x fastest, three components per point) and writes <prefix>_<numTS, 8 digits>.vtr.
//      A full pool of host buffers makes the host wait for the writer (back pressure).
// The file holds the dump's sample coordinates as Float64 x/y/z arrays and the field as a Float32
// vector array named "E-Field" or "H-Field" (ProcessFields::GetFieldNameByType), in raw appended
// binary (uncompressed; the reference compresses with zlib, which readers handle either way).
#include <cuda_runtime.h>

#include <algorithm>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <cmath>
#include <complex>
#include <vector>

#include "engine_impl.h"

namespace {

struct TdBuf {
    float* host = nullptr;      // pinned, float [3][npos]
    cudaEvent_t ev = nullptr;   // the copy into it completed
};

struct TdDump {
    int index = 0;                       // into e->dump_dev
    int field = 0;
    unsigned interval = 1, start = 0, stop = 0xFFFFFFFFu, nslot = 1, npos = 0, sz[3] = {0, 0, 0};
    const float* ring = nullptr;
    std::string prefix;
    std::vector<double> coords;          // x, y, z
    unsigned long long next_ts = 0;      // first step whose sample is not yet handed to the writer
    std::vector<int> free_bufs;
    std::vector<TdBuf> bufs;
};

struct Job {
    int dump;
    unsigned ts;
    int buf;
};

bool is_sample(const TdDump& d, unsigned long long ts)
{
    return ts >= d.start && ts <= d.stop && ts % d.interval == 0;
}

// samples of dump d at the steps (t, t + m]
unsigned samples_in(const TdDump& d, unsigned long long t, unsigned m)
{
    unsigned c = 0;
    for (unsigned long long s = t + 1; s <= t + m; ++s) c += is_sample(d, s);
    return c;
}

}  // namespace

struct oems_td_pipeline {
    int device = 0;
    std::vector<TdDump> dumps;
    std::mutex m;
    std::condition_variable cv;      // new jobs, finished jobs, freed buffers
    std::deque<Job> jobs;
    unsigned busy = 0;               // jobs the writer has taken and not finished
    bool stop = false;
    int error = 0;
    std::string errmsg;
    std::thread writer;
};

namespace {

// a vector field float [3][sx][sy][sz] (z fastest) on a rectilinear grid as a VTK XML
// RectilinearGrid file (raw appended data, UInt64 block headers); coords = x, y, z lines
int write_vtr_file(const std::string& path, const char* name, const unsigned dims[3], const double* coords,
                   const float* data, std::string& err)
{
    const unsigned sx = dims[0], sy = dims[1], sz = dims[2];
    const size_t npos = (size_t)sx * sy * sz;
    const uint16_t probe = 1;
    unsigned char lo;
    std::memcpy(&lo, &probe, 1);
    const char* order = lo ? "LittleEndian" : "BigEndian";
    const uint64_t nf = 12ull * npos, nx = 8ull * sx, ny = 8ull * sy, nz = 8ull * sz;
    const uint64_t off_x = 8 + nf, off_y = off_x + 8 + nx, off_z = off_y + 8 + ny;
    char head[2048];
    const int hl = std::snprintf(
        head, sizeof(head),
        "<?xml version=\"1.0\"?>\n"
        "<VTKFile type=\"RectilinearGrid\" version=\"1.0\" byte_order=\"%s\" header_type=\"UInt64\">\n"
        "  <RectilinearGrid WholeExtent=\"0 %u 0 %u 0 %u\">\n"
        "    <Piece Extent=\"0 %u 0 %u 0 %u\">\n"
        "      <PointData Vectors=\"%s\">\n"
        "        <DataArray type=\"Float32\" Name=\"%s\" NumberOfComponents=\"3\" format=\"appended\" offset=\"0\"/>\n"
        "      </PointData>\n"
        "      <CellData>\n"
        "      </CellData>\n"
        "      <Coordinates>\n"
        "        <DataArray type=\"Float64\" Name=\"x\" format=\"appended\" offset=\"%llu\"/>\n"
        "        <DataArray type=\"Float64\" Name=\"y\" format=\"appended\" offset=\"%llu\"/>\n"
        "        <DataArray type=\"Float64\" Name=\"z\" format=\"appended\" offset=\"%llu\"/>\n"
        "      </Coordinates>\n"
        "    </Piece>\n"
        "  </RectilinearGrid>\n"
        "  <AppendedData encoding=\"raw\">\n"
        "   _",
        order, sx - 1, sy - 1, sz - 1, sx - 1, sy - 1, sz - 1, name, name, (unsigned long long)off_x,
        (unsigned long long)off_y, (unsigned long long)off_z);
    if (hl <= 0 || hl >= (int)sizeof(head)) {
        err = "VTK header too long";
        return OEMS_ERR_IO;
    }
    // the sample is [3][sx][sy][sz] with z fastest; VTK points run x fastest
    std::vector<float> pts(3 * npos);
    for (unsigned k = 0; k < sz; ++k)
        for (unsigned j = 0; j < sy; ++j)
            for (unsigned i = 0; i < sx; ++i) {
                const size_t q = ((size_t)i * sy + j) * sz + k;
                const size_t p = ((size_t)k * sy + j) * sx + i;
                pts[3 * p] = data[q];
                pts[3 * p + 1] = data[npos + q];
                pts[3 * p + 2] = data[2 * npos + q];
            }
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) {
        err = "cannot open " + path;
        return OEMS_ERR_IO;
    }
    bool ok = std::fwrite(head, 1, (size_t)hl, f) == (size_t)hl;
    auto block = [&](const void* p, uint64_t n) {
        ok = ok && std::fwrite(&n, 8, 1, f) == 1;
        ok = ok && (n == 0 || std::fwrite(p, 1, (size_t)n, f) == (size_t)n);
    };
    block(pts.data(), nf);
    block(coords, nx);
    block(coords + sx, ny);
    block(coords + sx + sy, nz);
    const char* tail = "\n  </AppendedData>\n</VTKFile>\n";
    ok = ok && std::fwrite(tail, 1, std::strlen(tail), f) == std::strlen(tail);
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) {
        err = "write failed: " + path;
        return OEMS_ERR_IO;
    }
    return OEMS_OK;
}

// one time-domain sample: <prefix>_<numTS, 8 digits>.vtr
int write_vtr(const TdDump& d, unsigned ts, const float* data, std::string& err)
{
    char tsbuf[32];
    std::snprintf(tsbuf, sizeof(tsbuf), "%08u", ts);
    return write_vtr_file(d.prefix + "_" + tsbuf + ".vtr", d.field == 0 ? "E-Field" : "H-Field", d.sz,
                          d.coords.data(), data, err);
}

void writer_loop(oems_td_pipeline* p)
{
    cudaSetDevice(p->device);
    for (;;) {
        Job j;
        {
            std::unique_lock<std::mutex> lk(p->m);
            p->cv.wait(lk, [&] { return p->stop || !p->jobs.empty(); });
            if (p->jobs.empty()) break;   // stop requested and nothing left
            j = p->jobs.front();
            p->jobs.pop_front();
            ++p->busy;
        }
        TdDump& d = p->dumps[j.dump];
        TdBuf& b = d.bufs[j.buf];
        std::string err;
        int rc = OEMS_OK;
        const cudaError_t c = cudaEventSynchronize(b.ev);
        if (c != cudaSuccess) {
            rc = OEMS_ERR_CUDA;
            err = std::string("time-domain dump copy: ") + cudaGetErrorString(c);
        } else {
            rc = write_vtr(d, j.ts, b.host, err);
        }
        {
            std::lock_guard<std::mutex> lk(p->m);
            if (rc && !p->error) {
                p->error = rc;
                p->errmsg = err;
            }
            d.free_bufs.push_back(j.buf);
            --p->busy;
        }
        p->cv.notify_all();
    }
}

}  // namespace

int td_start_pipeline(oems_cuda_engine* e)
{
    auto* p = new (std::nothrow) oems_td_pipeline();
    if (!p) return OEMS_ERR_NOMEM;
    e->td = p;
    p->device = e->device;
    for (size_t k = 0; k < e->dumps.size(); ++k) {
        const DumpHost& h = e->dumps[k];
        if (!h.td) continue;
        const DumpDev& dd = e->dump_dev[k];
        TdDump d;
        d.index = (int)k;
        d.field = h.field;
        d.interval = h.td_interval;
        d.start = h.td_start;
        d.stop = h.td_stop;
        d.nslot = dd.nslot;
        d.npos = dd.npos;
        for (int a = 0; a < 3; ++a) d.sz[a] = dd.sz[a];
        d.ring = dd.ring;
        d.prefix = h.prefix;
        d.coords = h.coords;
        // pinned host buffers: up to 4 samples in flight within about 1 GB
        const size_t bytes = 12ull * d.npos;
        const size_t nbuf = std::min<size_t>(4, std::max<size_t>(1, (size_t(1) << 30) / bytes));
        for (size_t b = 0; b < nbuf; ++b) {
            TdBuf tb;
            if (cudaHostAlloc((void**)&tb.host, bytes, cudaHostAllocDefault) != cudaSuccess) {
                e->err = "time-domain dump: pinned host buffer allocation failed";
                d.bufs.push_back(tb);
                p->dumps.push_back(std::move(d));
                return OEMS_ERR_NOMEM;
            }
            if (cudaEventCreateWithFlags(&tb.ev, cudaEventDisableTiming) != cudaSuccess) {
                d.bufs.push_back(tb);
                p->dumps.push_back(std::move(d));
                e->err = "time-domain dump: event creation failed";
                return OEMS_ERR_CUDA;
            }
            d.free_bufs.push_back((int)d.bufs.size());
            d.bufs.push_back(tb);
        }
        p->dumps.push_back(std::move(d));
    }
    p->writer = std::thread(writer_loop, p);
    return OEMS_OK;
}

int td_flush(oems_cuda_engine* e)
{
    oems_td_pipeline* p = e->td;
    if (!p) return OEMS_OK;
    const unsigned long long now = e->host_numTS;
    for (size_t k = 0; k < p->dumps.size(); ++k) {
        TdDump& d = p->dumps[k];
        // the first sample step at or after next_ts
        unsigned long long ts = std::max<unsigned long long>(d.next_ts, d.start);
        ts = (ts + d.interval - 1) / d.interval * d.interval;
        for (; ts <= now && ts <= d.stop; ts += d.interval) {
            int b;
            {
                std::unique_lock<std::mutex> lk(p->m);
                p->cv.wait(lk, [&] { return !d.free_bufs.empty(); });
                b = d.free_bufs.back();
                d.free_bufs.pop_back();
            }
            TdBuf& tb = d.bufs[b];
            const float* slot = d.ring + (size_t)((ts / d.interval) % d.nslot) * 3 * d.npos;
            cudaError_t c = cudaMemcpyAsync(tb.host, slot, 12ull * d.npos, cudaMemcpyDeviceToHost, e->stream);
            if (c == cudaSuccess) c = cudaEventRecord(tb.ev, e->stream);
            if (c != cudaSuccess) {
                std::lock_guard<std::mutex> lk(p->m);
                d.free_bufs.push_back(b);
                e->err = std::string("time-domain dump copy: ") + cudaGetErrorString(c);
                return OEMS_ERR_CUDA;
            }
            {
                std::lock_guard<std::mutex> lk(p->m);
                p->jobs.push_back(Job{(int)k, (unsigned)ts, b});
            }
            p->cv.notify_all();
        }
        d.next_ts = now + 1;
    }
    return OEMS_OK;
}

int td_iterate(oems_cuda_engine* e, unsigned n)
{
    oems_td_pipeline* p = e->td;
    unsigned long long t = e->host_numTS;
    const unsigned long long end = t + n;
    std::vector<unsigned> pending(p ? p->dumps.size() : 0, 0);
    while (t < end) {
        unsigned m = (end - t >= e->K) ? e->K : 1;
        if (p) {
            // a K-step replay must fit every dump's ring; else single steps
            for (const auto& d : p->dumps)
                if (m > 1 && samples_in(d, t, m) > d.nslot) m = 1;
            bool flush = false;
            for (size_t k = 0; k < p->dumps.size(); ++k)
                flush = flush || pending[k] + samples_in(p->dumps[k], t, m) > p->dumps[k].nslot;
            if (flush) {
                int rc = td_flush(e);
                if (rc) return rc;
                std::fill(pending.begin(), pending.end(), 0u);
            }
            for (size_t k = 0; k < p->dumps.size(); ++k) pending[k] += samples_in(p->dumps[k], t, m);
        }
        const cudaError_t c = cudaGraphLaunch(m == e->K ? e->graphK : e->graph1, e->stream);
        if (c != cudaSuccess) {
            e->err = std::string("cudaGraphLaunch: ") + cudaGetErrorString(c);
            return OEMS_ERR_CUDA;
        }
        t += m;
        e->host_numTS = (unsigned)t;
    }
    return td_flush(e);
}

int td_wait(oems_cuda_engine* e)
{
    oems_td_pipeline* p = e->td;
    if (!p) return OEMS_OK;
    std::unique_lock<std::mutex> lk(p->m);
    p->cv.wait(lk, [&] { return p->jobs.empty() && p->busy == 0; });
    if (p->error) {
        e->err = p->errmsg;
        return p->error;
    }
    return OEMS_OK;
}

void td_free(oems_cuda_engine* e)
{
    oems_td_pipeline* p = e->td;
    if (!p) return;
    {
        std::lock_guard<std::mutex> lk(p->m);
        p->stop = true;
    }
    p->cv.notify_all();
    if (p->writer.joinable()) p->writer.join();
    for (auto& d : p->dumps)
        for (auto& b : d.bufs) {
            if (b.host) cudaFreeHost(b.host);
            if (b.ev) cudaEventDestroy(b.ev);
        }
    delete p;
    e->td = nullptr;
}

// ProcessFieldsFD::DumpFDData for the VTK file type (Common/processfields_fd.cpp:114-215): per
// frequency, 21 phase snapshots real(F * exp(j * 2 pi p / 21)), the magnitude |F| and the phase
// arg(F) of every component, as <prefix>_f=<freq>_p=<degrees, 3 digits>.vtr, ..._abs.vtr and
// ..._arg.vtr.  The frequency is written as an integer when it is one, else with six decimals
// (std::to_string), and the arithmetic is the reference's complex<float> arithmetic.
extern "C" int oems_cuda_write_fd_dump(oems_cuda_engine* e, int id, const char* prefix, const double* coords)
{
    if (!e || !prefix || !prefix[0] || !coords || id < 0 || id >= (int)e->dumps.size()) return OEMS_ERR_ARG;
    if (!e->inited) return OEMS_ERR_STATE;
    const DumpHost& h = e->dumps[id];
    if (h.td) return OEMS_ERR_ARG;
    unsigned dims[3];
    size_t npos = 1;
    for (int a = 0; a < 3; ++a) {
        dims[a] = h.stop[a] - h.start[a] + 1;
        npos *= dims[a];
    }
    const size_t nf = h.freqs.size();
    std::vector<float> acc(nf * 3 * npos * 2);
    int rc = oems_cuda_read_fd_dump(e, id, acc.data(), acc.size());
    if (rc != OEMS_OK) return rc;
    const char* name = h.field == 0 ? "E-Field" : "H-Field";
    std::vector<float> out(3 * npos);
    std::string err;
    const int Nr_Ph = 21;
    for (size_t f = 0; f < nf; ++f) {
        const double freq = h.freqs[f];
        const std::string sf = (freq - (long)freq) == 0 ? std::to_string((long)freq) : std::to_string(freq);
        const std::complex<float>* F = reinterpret_cast<const std::complex<float>*>(acc.data()) + f * 3 * npos;
        for (int p = 0; p < Nr_Ph; ++p) {
            const double angle = 2.0 * M_PI * p / Nr_Ph;
            const std::complex<float> ejw = std::exp((std::complex<float>)(std::complex<double>(0.0, 1.0) * angle));
            for (size_t q = 0; q < 3 * npos; ++q) out[q] = std::real(F[q] * ejw);
            char deg[16];
            std::snprintf(deg, sizeof(deg), "%03d", (int)(angle * 180 / M_PI));
            rc = write_vtr_file(std::string(prefix) + "_f=" + sf + "_p=" + deg + ".vtr", name, dims, coords, out.data(), err);
            if (rc != OEMS_OK) { e->err = err; return rc; }
        }
        for (size_t q = 0; q < 3 * npos; ++q) out[q] = std::abs(F[q]);
        rc = write_vtr_file(std::string(prefix) + "_f=" + sf + "_abs.vtr", name, dims, coords, out.data(), err);
        if (rc != OEMS_OK) { e->err = err; return rc; }
        for (size_t q = 0; q < 3 * npos; ++q) out[q] = std::arg(F[q]);
        rc = write_vtr_file(std::string(prefix) + "_f=" + sf + "_arg.vtr", name, dims, coords, out.data(), err);
        if (rc != OEMS_OK) { e->err = err; return rc; }
    }
    return OEMS_OK;
}
