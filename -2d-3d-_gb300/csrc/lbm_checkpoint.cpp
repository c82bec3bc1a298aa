// lbm_checkpoint.cpp - Fortran unformatted sequential records, the reference's restart
// file format.
//
// backupData (3DRB.F90:1638-1665, 2DRB.F90:1402-1430) writes two records,
// ((((f(alpha,i,j,k),i=1,nx),j=1,ny),k=1,nz),alpha=0,qf-1) and the same for g, that
// loadInitField = 1 reads back (3DRB.F90:602-623, 2DRB.F90:621-637).  gfortran frames a
// record as [int32 n][n bytes][int32 n]; a record longer than 2^31 - 9 bytes is split into
// subrecords, every subrecord but the last with a negative leading marker and every
// subrecord but the first with a negative trailing marker.  Markers are little-endian on
// both machines this library builds for.
#include <cstring>

#include "../../include/lbm_gpu.h"
#include "lbm_records.h"

namespace lbm {

namespace {
size_t g_limit = kMaxSubrecord;

bool put_marker(FILE* fp, int32_t m) { return std::fwrite(&m, 4, 1, fp) == 1; }
bool get_marker(FILE* fp, int32_t* m) { return std::fread(m, 4, 1, fp) == 1; }
}  // namespace

size_t subrecord_limit() { return g_limit; }

bool RecordWriter::begin(FILE* f, size_t total) {
    fp = f;
    left = total;
    first = true;
    ok = fp != nullptr;
    sub_left = 0;
    if (!ok) return false;
    // open the first subrecord (also for an empty record)
    sub_len = left > g_limit ? g_limit : left;
    sub_left = sub_len;
    const bool last = left == sub_len;
    ok = put_marker(fp, last ? (int32_t)sub_len : -(int32_t)sub_len);
    return ok;
}

bool RecordWriter::put(const void* data, size_t n) {
    const unsigned char* p = (const unsigned char*)data;
    while (ok && n > 0) {
        if (sub_left == 0) {
            // close the current subrecord, open the next
            ok = put_marker(fp, first ? (int32_t)sub_len : -(int32_t)sub_len);
            first = false;
            if (!ok) break;
            sub_len = left > g_limit ? g_limit : left;
            sub_left = sub_len;
            const bool last = left == sub_len;
            if (sub_len == 0) {
                ok = false;  // more data than announced
                break;
            }
            ok = put_marker(fp, last ? (int32_t)sub_len : -(int32_t)sub_len);
            if (!ok) break;
        }
        const size_t k = n < sub_left ? n : sub_left;
        if (k > left || std::fwrite(p, 1, k, fp) != k) {
            ok = false;
            break;
        }
        p += k;
        n -= k;
        sub_left -= k;
        left -= k;
    }
    return ok;
}

bool RecordWriter::end() {
    if (!ok || left != 0 || sub_left != 0) return ok = false;
    ok = put_marker(fp, first ? (int32_t)sub_len : -(int32_t)sub_len);
    return ok;
}

bool RecordReader::begin(FILE* f) {
    fp = f;
    total = 0;
    ok = fp != nullptr;
    open = false;
    if (!ok) return false;
    int32_t m = 0;
    if (!get_marker(fp, &m)) return ok = false;
    more = m < 0;
    sub_len = (size_t)(m < 0 ? -(int64_t)m : m);
    sub_left = sub_len;
    open = true;
    return true;
}

size_t RecordReader::get(void* dst, size_t n) {
    unsigned char* p = (unsigned char*)dst;
    size_t got = 0;
    while (ok && open && got < n) {
        if (sub_left == 0) {
            int32_t t = 0;
            if (!get_marker(fp, &t) || (size_t)(t < 0 ? -(int64_t)t : t) != sub_len) {
                ok = false;
                break;
            }
            if (!more) {
                open = false;
                break;
            }
            int32_t m = 0;
            if (!get_marker(fp, &m)) {
                ok = false;
                break;
            }
            more = m < 0;
            sub_len = (size_t)(m < 0 ? -(int64_t)m : m);
            sub_left = sub_len;
            continue;
        }
        const size_t k = (n - got) < sub_left ? (n - got) : sub_left;
        if (std::fread(p + got, 1, k, fp) != k) {
            ok = false;
            break;
        }
        got += k;
        sub_left -= k;
        total += k;
    }
    // close the record if its last byte was just delivered
    if (ok && open && sub_left == 0 && !more) {
        int32_t t = 0;
        if (!get_marker(fp, &t) || (size_t)(t < 0 ? -(int64_t)t : t) != sub_len) ok = false;
        open = false;
    }
    return got;
}

bool RecordReader::skip_rest() {
    while (ok && open) {
        if (sub_left > 0) {
            if (std::fseek(fp, (long)sub_left, SEEK_CUR) != 0) return ok = false;
            total += sub_left;
            sub_left = 0;
        }
        int32_t t = 0;
        if (!get_marker(fp, &t) || (size_t)(t < 0 ? -(int64_t)t : t) != sub_len) return ok = false;
        if (!more) {
            open = false;
            break;
        }
        int32_t m = 0;
        if (!get_marker(fp, &m)) return ok = false;
        more = m < 0;
        sub_len = (size_t)(m < 0 ? -(int64_t)m : m);
        sub_left = sub_len;
    }
    return ok;
}

}  // namespace lbm

using namespace lbm;

extern "C" int lbm_fortran_set_subrecord_limit(size_t max_subrecord_bytes) {
    if (max_subrecord_bytes < 1 || max_subrecord_bytes > kMaxSubrecord) return LBM_ERR_PARAM;
    g_limit = max_subrecord_bytes;
    return LBM_OK;
}

extern "C" int lbm_fortran_record_write(const char* path, int append, const void* data, size_t nbytes) {
    if (!path || (!data && nbytes)) return LBM_ERR_PARAM;
    FILE* fp = std::fopen(path, append ? "ab" : "wb");
    if (!fp) return LBM_ERR_IO;
    RecordWriter w;
    bool ok = w.begin(fp, nbytes) && w.put(data, nbytes) && w.end();
    if (std::fclose(fp) != 0) ok = false;
    return ok ? LBM_OK : LBM_ERR_IO;
}

extern "C" int lbm_fortran_record_read(const char* path, uint64_t offset, void* data, size_t capacity,
                                       size_t* nbytes, uint64_t* next_offset) {
    if (!path || !nbytes || (!data && capacity)) return LBM_ERR_PARAM;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return LBM_ERR_IO;
    int st = LBM_OK;
    RecordReader r;
    if (std::fseek(fp, (long)offset, SEEK_SET) != 0 || !r.begin(fp)) {
        st = LBM_ERR_IO;
    } else {
        if (capacity) r.get(data, capacity);
        const size_t delivered = r.total;
        if (!r.skip_rest()) st = LBM_ERR_IO;
        *nbytes = r.total;
        if (st == LBM_OK && r.total > delivered) st = LBM_ERR_TOO_LARGE;  // record longer than the buffer
        if (next_offset) *next_offset = (uint64_t)std::ftell(fp);
    }
    std::fclose(fp);
    return st;
}
