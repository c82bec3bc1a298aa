// lbm_records.h - streaming reader and writer of Fortran unformatted sequential records
// (gfortran layout, 4-byte markers, subrecords for records above 2 GiB).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstdio>

namespace lbm {

// Largest subrecord payload gfortran writes: 2^31 - 9 bytes.
constexpr size_t kMaxSubrecord = 2147483639u;
size_t subrecord_limit();

// Writes one logical record of a length known in advance, in pieces.
struct RecordWriter {
    FILE* fp = nullptr;
    size_t left = 0;      // bytes of the record still to come
    size_t sub_left = 0;  // bytes of the open subrecord still to come
    size_t sub_len = 0;
    bool first = true;
    bool ok = true;
    bool begin(FILE* f, size_t total);
    bool put(const void* data, size_t n);
    bool end();  // true iff every byte was written and the markers are closed
};

// Reads one logical record in pieces; the total length is known only at the end.
struct RecordReader {
    FILE* fp = nullptr;
    size_t sub_left = 0;
    size_t sub_len = 0;
    bool more = false;    // another subrecord follows the open one
    bool open = false;
    bool ok = true;
    size_t total = 0;     // bytes delivered so far
    bool begin(FILE* f);
    size_t get(void* dst, size_t n);  // returns the bytes delivered (< n at the record's end)
    bool skip_rest();                 // skip to the end of the record
    bool at_end() const { return !open; }
};

}  // namespace lbm
