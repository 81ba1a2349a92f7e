// Snapshots of device or host arrays (orbital blocks, potentials, learned
// weights) in one flat file: MGmol's restart role (MGmol::dumpRestart with
// HDFrestart, src/MGmol.cc:1101-1127, src/HDFrestart.cc) without the HDF5
// library, which is not available to this build.
//
// File layout (little-endian):
//   [0, 8)    magic "MGXSNAP1"
//   [8, 16)   header length H (bytes of JSON)
//   [16, 24)  offset of the first array (a multiple of 4096)
//   [24, 64)  zero
//   [64, 64+H) JSON header: {"format":"mgx-snapshot","version":1,
//             "grid":{"n":[..],"ll":[..]},"meta":<caller's JSON or null>,
//             "datasets":[{"name":..,"type":"f64"|"f32"|"i32"|"u8",
//             "shape":[..],"offset":..,"bytes":..,"crc32":"0x........"},..]}
//   then each array's raw bytes at its offset (4096-aligned).
// Arrays move through two pinned host buffers: the device-to-host copy of
// one 64 MiB chunk overlaps the file write of the previous one, and the
// CRC-32 of each array is accumulated on the way and checked on reading.
#include <cuda_runtime.h>

#include <cerrno>
#include <algorithm>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mgx_internal.cuh"

namespace mgx
{
namespace
{
constexpr size_t SNAP_ALIGN = 4096;
constexpr size_t SNAP_CHUNK = size_t(64) << 20;
constexpr size_t SNAP_FIXED = 64;

struct CrcTable
{
    uint32_t t[256];
    CrcTable()
    {
        for (uint32_t i = 0; i < 256; i++)
        {
            uint32_t c = i;
            for (int k = 0; k < 8; k++)
                c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
    }
};

/* CRC-32 (IEEE 802.3, reflected polynomial 0xEDB88320) continued over
 * [p, p + n) */
uint32_t crc_update(uint32_t crc, const unsigned char* p, size_t n)
{
    static const CrcTable table; // initialized once, thread-safe
    crc = ~crc;
    for (size_t i = 0; i < n; i++)
        crc = table.t[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return ~crc;
}

size_t type_bytes(int t)
{
    switch (t)
    {
        case MGX_SNAP_F64: return 8;
        case MGX_SNAP_F32: return 4;
        case MGX_SNAP_I32: return 4;
        case MGX_SNAP_U8: return 1;
    }
    return 0;
}
const char* type_name(int t)
{
    switch (t)
    {
        case MGX_SNAP_F64: return "f64";
        case MGX_SNAP_F32: return "f32";
        case MGX_SNAP_I32: return "i32";
        case MGX_SNAP_U8: return "u8";
    }
    return "?";
}

/* device memory (or managed) that the host cannot read directly */
bool on_device(const void* p)
{
    cudaPointerAttributes a;
    const cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice;
}

/* two staging buffers, pinned when a device is present */
struct Staging
{
    void* buf[2]  = { nullptr, nullptr };
    bool pinned   = false;
    ~Staging()
    {
        for (void* b : buf)
            if (b)
            {
                if (pinned)
                    cudaFreeHost(b);
                else
                    free(b);
            }
    }
    int init()
    {
        pinned = true;
        for (void*& b : buf)
            if (cudaMallocHost(&b, SNAP_CHUNK) != cudaSuccess)
            {
                cudaGetLastError();
                pinned = false;
                break;
            }
        if (!pinned)
        {
            for (void*& b : buf)
                if (b)
                {
                    cudaFreeHost(b);
                    b = nullptr;
                }
            for (void*& b : buf)
                if (!(b = malloc(SNAP_CHUNK))) return fail(MGX_NO_MEMORY, "snapshot staging buffer");
        }
        return MGX_OK;
    }
};

std::string header_json(const mgx_grid* g, const char* meta, int n, const mgx_dataset* d,
    const std::vector<size_t>& off, const std::vector<uint32_t>& crc)
{
    std::string s = "{\"format\":\"mgx-snapshot\",\"version\":1,\"grid\":";
    char buf[512];
    if (g)
    {
        snprintf(buf, sizeof(buf), "{\"n\":[%d,%d,%d],\"ll\":[%.17g,%.17g,%.17g]}", g->n[0], g->n[1],
            g->n[2], g->ll[0], g->ll[1], g->ll[2]);
        s += buf;
    }
    else
        s += "null";
    s += ",\"meta\":";
    s += (meta && *meta) ? meta : "null";
    s += ",\"datasets\":[";
    for (int i = 0; i < n; i++)
    {
        if (i) s += ",";
        s += "{\"name\":\"";
        s += d[i].name;
        s += "\",\"type\":\"";
        s += type_name(d[i].type);
        s += "\",\"shape\":[";
        size_t bytes = type_bytes(d[i].type);
        for (int k = 0; k < d[i].ndim; k++)
        {
            snprintf(buf, sizeof(buf), "%s%zu", k ? "," : "", d[i].shape[k]);
            s += buf;
            bytes *= d[i].shape[k];
        }
        snprintf(buf, sizeof(buf), "],\"offset\":%zu,\"bytes\":%zu,\"crc32\":\"0x%08" PRIx32 "\"}",
            off[i], bytes, crc[i]);
        s += buf;
    }
    s += "]}";
    return s;
}

int check_name(const char* nm)
{
    if (!nm || !*nm) return fail(MGX_BAD_ARG, "snapshot dataset without a name");
    for (const char* c = nm; *c; c++)
        if (*c == '"' || *c == '\\' || (unsigned char)*c < 0x20)
            return fail(MGX_BAD_ARG, "snapshot dataset name '%s' has a character JSON would escape", nm);
    return MGX_OK;
}

/* the fields of dataset `name` from a header this file wrote */
int find_dataset(const std::string& h, const char* name, size_t* off, size_t* bytes,
    uint32_t* crc)
{
    const std::string key = std::string("{\"name\":\"") + name + "\",";
    const size_t p        = h.find(key);
    if (p == std::string::npos) return fail(MGX_BAD_ARG, "snapshot has no dataset '%s'", name);
    const size_t po = h.find("\"offset\":", p), pb = h.find("\"bytes\":", p),
                 pc = h.find("\"crc32\":\"", p);
    if (po == std::string::npos || pb == std::string::npos || pc == std::string::npos)
        return fail(MGX_BAD_ARG, "snapshot header of '%s' is malformed", name);
    *off   = (size_t)strtoull(h.c_str() + po + 9, nullptr, 10);
    *bytes = (size_t)strtoull(h.c_str() + pb + 8, nullptr, 10);
    *crc   = (uint32_t)strtoul(h.c_str() + pc + 9, nullptr, 16);
    return MGX_OK;
}

int read_header(FILE* f, std::string& h, size_t* data_off)
{
    unsigned char fixed[SNAP_FIXED];
    if (fread(fixed, 1, SNAP_FIXED, f) != SNAP_FIXED || memcmp(fixed, "MGXSNAP1", 8) != 0)
        return fail(MGX_BAD_ARG, "not an mgx snapshot");
    uint64_t hl = 0, d0 = 0;
    memcpy(&hl, fixed + 8, 8);
    memcpy(&d0, fixed + 16, 8);
    if (hl == 0 || hl > (uint64_t(64) << 20)) return fail(MGX_BAD_ARG, "snapshot header length %llu", (unsigned long long)hl);
    h.resize((size_t)hl);
    if (fread(&h[0], 1, (size_t)hl, f) != (size_t)hl) return fail(MGX_BAD_ARG, "snapshot header truncated");
    if (data_off) *data_off = (size_t)d0;
    return MGX_OK;
}
} // namespace
} // namespace mgx

using namespace mgx;

extern "C" int mgx_snapshot_write(const char* path, const mgx_grid* grid, const char* meta_json,
    int ndata, const mgx_dataset* data, void* stream)
{
    if (!path || ndata < 0 || (ndata > 0 && !data)) return fail(MGX_BAD_ARG, "snapshot: null argument");
    std::vector<size_t> off(ndata), nbytes(ndata);
    std::vector<uint32_t> crc(ndata, 0u);
    for (int i = 0; i < ndata; i++)
    {
        MGX_TRY(check_name(data[i].name));
        for (int j = 0; j < i; j++)
            if (strcmp(data[i].name, data[j].name) == 0)
                return fail(MGX_BAD_ARG, "snapshot dataset '%s' appears twice", data[i].name);
        if (type_bytes(data[i].type) == 0) return fail(MGX_BAD_ARG, "snapshot type %d", data[i].type);
        if (data[i].ndim < 0 || data[i].ndim > 4) return fail(MGX_BAD_ARG, "snapshot ndim %d", data[i].ndim);
        nbytes[i] = type_bytes(data[i].type);
        for (int k = 0; k < data[i].ndim; k++)
            nbytes[i] *= data[i].shape[k];
        if (nbytes[i] && !data[i].data) return fail(MGX_BAD_ARG, "snapshot dataset '%s' has no data", data[i].name);
    }
    // the header with placeholder checksums has its final length
    std::string h = header_json(grid, meta_json, ndata, data, off, crc);
    size_t pos    = (SNAP_FIXED + h.size() + 2 * 64 * ndata + SNAP_ALIGN - 1) / SNAP_ALIGN * SNAP_ALIGN;
    const size_t d0 = pos;
    for (int i = 0; i < ndata; i++)
    {
        off[i] = pos;
        pos += (nbytes[i] + SNAP_ALIGN - 1) / SNAP_ALIGN * SNAP_ALIGN;
    }
    h = header_json(grid, meta_json, ndata, data, off, crc);
    if (SNAP_FIXED + h.size() > d0) return fail(MGX_BAD_ARG, "snapshot header grew past its room");

    FILE* f = fopen(path, "wb");
    if (!f) return fail(MGX_BAD_ARG, "snapshot: cannot open %s for writing: %s", path, strerror(errno));
    Staging st;
    int rc = st.init();
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char fixed[SNAP_FIXED] = {};
    memcpy(fixed, "MGXSNAP1", 8);
    const uint64_t hl = h.size(), dd = d0;
    memcpy(fixed + 8, &hl, 8);
    memcpy(fixed + 16, &dd, 8);
    if (rc == MGX_OK && (fwrite(fixed, 1, SNAP_FIXED, f) != SNAP_FIXED || fwrite(h.data(), 1, h.size(), f) != h.size()))
        rc = fail(MGX_BAD_ARG, "snapshot: write of %s failed", path);
    for (int i = 0; rc == MGX_OK && i < ndata; i++)
    {
        if (fseek(f, (long)off[i], SEEK_SET) != 0)
        {
            rc = fail(MGX_BAD_ARG, "snapshot: seek in %s failed", path);
            break;
        }
        const unsigned char* src = (const unsigned char*)data[i].data;
        const bool dev           = nbytes[i] && on_device(src);
        // chunk k is copied into buffer k % 2 while chunk k - 1 is written
        size_t done = 0;
        int k       = 0;
        size_t pending = 0;
        while (rc == MGX_OK && (done < nbytes[i] || pending))
        {
            const size_t n = std::min(SNAP_CHUNK, nbytes[i] - done);
            unsigned char* b = (unsigned char*)st.buf[k % 2];
            if (n)
            {
                if (dev)
                    rc = cuda_check(cudaMemcpyAsync(b, src + done, n, cudaMemcpyDeviceToHost, s), "snapshot copy");
                else
                    memcpy(b, src + done, n);
            }
            if (rc == MGX_OK && pending)
            {
                unsigned char* pb = (unsigned char*)st.buf[(k + 1) % 2];
                crc[i]            = crc_update(crc[i], pb, pending);
                if (fwrite(pb, 1, pending, f) != pending) rc = fail(MGX_BAD_ARG, "snapshot: write of %s failed", path);
            }
            if (rc == MGX_OK && dev && n) rc = cuda_check(cudaStreamSynchronize(s), "snapshot copy");
            done += n;
            pending = n;
            k++;
        }
    }
    if (rc == MGX_OK)
    {
        h = header_json(grid, meta_json, ndata, data, off, crc);
        if (fseek(f, (long)SNAP_FIXED, SEEK_SET) != 0 || fwrite(h.data(), 1, h.size(), f) != h.size())
            rc = fail(MGX_BAD_ARG, "snapshot: header rewrite of %s failed", path);
        // the file ends on the last array's aligned end: a zero byte there
        // when that end lies past the data (never over the data itself)
        const size_t data_end = ndata ? off[ndata - 1] + nbytes[ndata - 1] : d0;
        if (rc == MGX_OK && pos > data_end
            && (fseek(f, (long)pos - 1, SEEK_SET) != 0 || fputc(0, f) == EOF))
            rc = fail(MGX_BAD_ARG, "snapshot: write of %s failed", path);
    }
    if (fclose(f) != 0 && rc == MGX_OK) rc = fail(MGX_BAD_ARG, "snapshot: close of %s failed", path);
    return rc;
}

extern "C" int mgx_snapshot_header(const char* path, char* json, size_t cap, size_t* len)
{
    if (!path) return fail(MGX_BAD_ARG, "snapshot: null path");
    FILE* f = fopen(path, "rb");
    if (!f) return fail(MGX_BAD_ARG, "snapshot: cannot open %s: %s", path, strerror(errno));
    std::string h;
    const int rc = read_header(f, h, nullptr);
    fclose(f);
    if (rc != MGX_OK) return rc;
    if (len) *len = h.size();
    if (json && cap)
    {
        const size_t n = std::min(cap - 1, h.size());
        memcpy(json, h.data(), n);
        json[n] = '\0';
        if (n < h.size()) return fail(MGX_BAD_ARG, "snapshot header needs %zu bytes", h.size() + 1);
    }
    return MGX_OK;
}

extern "C" int mgx_snapshot_read(const char* path, const char* name, void* dst, size_t bytes,
    void* stream)
{
    if (!path || !name || (bytes && !dst)) return fail(MGX_BAD_ARG, "snapshot: null argument");
    FILE* f = fopen(path, "rb");
    if (!f) return fail(MGX_BAD_ARG, "snapshot: cannot open %s: %s", path, strerror(errno));
    std::string h;
    size_t off = 0, nb = 0;
    uint32_t crc_ref = 0, crc = 0;
    int rc = read_header(f, h, nullptr);
    if (rc == MGX_OK) rc = find_dataset(h, name, &off, &nb, &crc_ref);
    if (rc == MGX_OK && nb != bytes)
        rc = fail(MGX_BAD_ARG, "snapshot dataset '%s' holds %zu bytes, the destination %zu", name, nb, bytes);
    if (rc == MGX_OK && fseek(f, (long)off, SEEK_SET) != 0) rc = fail(MGX_BAD_ARG, "snapshot: seek failed");
    Staging st;
    if (rc == MGX_OK) rc = st.init();
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* out = (unsigned char*)dst;
    const bool dev     = rc == MGX_OK && nb && on_device(out);
    // chunk k is read into buffer k % 2 while chunk k - 1 is copied out
    size_t done = 0;
    int k       = 0;
    while (rc == MGX_OK && done < nb)
    {
        const size_t n   = std::min(SNAP_CHUNK, nb - done);
        unsigned char* b = (unsigned char*)st.buf[k % 2];
        if (dev && k >= 2) rc = cuda_check(cudaStreamSynchronize(s), "snapshot copy");
        if (rc == MGX_OK && fread(b, 1, n, f) != n) rc = fail(MGX_BAD_ARG, "snapshot dataset '%s' truncated", name);
        if (rc != MGX_OK) break;
        crc = crc_update(crc, b, n);
        if (dev)
            rc = cuda_check(cudaMemcpyAsync(out + done, b, n, cudaMemcpyHostToDevice, s), "snapshot copy");
        else
            memcpy(out + done, b, n);
        done += n;
        k++;
    }
    if (rc == MGX_OK && dev) rc = cuda_check(cudaStreamSynchronize(s), "snapshot copy");
    fclose(f);
    if (rc == MGX_OK && crc != crc_ref)
        rc = fail(MGX_BAD_ARG, "snapshot dataset '%s': checksum 0x%08x, header says 0x%08x", name,
            crc, crc_ref);
    return rc;
}
