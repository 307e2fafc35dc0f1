// .trees files: a read-only reader of the kastore container that tskit
// writes them in (c/subprojects/kastore/kastore.c, read by
// tsk_table_collection_load, c/tskit/tables.c:11580-11830).  The container:
//   * a 64-byte header: the 8-byte magic "\211KAS\r\n\032\n", the format's
//     major and minor version (uint16 each), the number of items (uint32)
//     and the file size (uint64), all little-endian;
//   * one 64-byte descriptor per item: its type (one byte, 0..9: int8,
//     uint8, int16, uint16, int32, uint32, int64, uint64, float32, float64)
//     and the offsets and lengths of its key and array (uint64 each, at
//     bytes 8, 16, 24 and 32);
//   * the keys, packed one after another right after the descriptors;
//   * the arrays, each starting on an 8-byte boundary, ending the file.
// The whole file is read into host memory and checked against that layout;
// lookups return pointers into it.  Host code only.
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "tskit_gb300.h"

struct tsg_kastore {
    std::vector<unsigned char> bytes;
    struct Item {
        int type;
        std::string key;
        uint64_t array_start, array_len;
    };
    std::vector<Item> items;
};

namespace {

const unsigned char KAS_MAGIC[8] = { 0x89, 'K', 'A', 'S', '\r', '\n', 0x1a, '\n' };
constexpr int KAS_HEADER = 64;
constexpr int KAS_DESCRIPTOR = 64;
constexpr int KAS_NUM_TYPES = 10;
constexpr uint16_t KAS_VERSION_MAJOR = 1;

int type_size(int type)
{
    static const int sizes[KAS_NUM_TYPES] = { 1, 1, 2, 2, 4, 4, 8, 8, 4, 8 };
    return sizes[type];
}

template <typename T>
T read_le(const unsigned char *p)
{
    T v = 0;
    for (size_t i = 0; i < sizeof(T); i++) {
        v |= (T) ((T) p[i] << (8 * i));
    }
    return v;
}

}  // namespace

extern "C" {

int tsg_kastore_open(const char *path, tsg_kastore_t **out)
{
    *out = nullptr;
    FILE *f = std::fopen(path, "rb");
    if (f == nullptr) {
        return TSG_ERR_IO;
    }
    auto *k = new (std::nothrow) tsg_kastore_t();
    if (k == nullptr) {
        std::fclose(f);
        return TSG_ERR_NO_MEMORY;
    }
    int ret = 0;
    unsigned char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) {
        k->bytes.insert(k->bytes.end(), chunk, chunk + got);
    }
    if (std::ferror(f)) {
        ret = TSG_ERR_IO;
    }
    std::fclose(f);
    const unsigned char *b = k->bytes.data();
    const uint64_t size = k->bytes.size();
    if (ret == 0 && (size < (uint64_t) KAS_HEADER || std::memcmp(b, KAS_MAGIC, 8) != 0)) {
        ret = TSG_ERR_FILE_FORMAT;
    }
    uint32_t num_items = 0;
    if (ret == 0) {
        const uint16_t major = read_le<uint16_t>(b + 8);
        num_items = read_le<uint32_t>(b + 12);
        const uint64_t file_size = read_le<uint64_t>(b + 16);
        if (major < KAS_VERSION_MAJOR) {
            ret = TSG_ERR_FILE_VERSION_TOO_OLD;
        } else if (major > KAS_VERSION_MAJOR) {
            ret = TSG_ERR_FILE_VERSION_TOO_NEW;
        } else if (file_size != size
            || (uint64_t) KAS_HEADER + (uint64_t) num_items * KAS_DESCRIPTOR > size) {
            ret = TSG_ERR_FILE_FORMAT;
        }
    }
    // descriptors, then the packing: keys right after the descriptors, arrays
    // 8-byte aligned and adjacent up to the end of the file
    uint64_t offset = (uint64_t) KAS_HEADER + (uint64_t) num_items * KAS_DESCRIPTOR;
    for (uint32_t j = 0; ret == 0 && j < num_items; j++) {
        const unsigned char *d = b + KAS_HEADER + (uint64_t) j * KAS_DESCRIPTOR;
        const int type = d[0];
        const uint64_t key_start = read_le<uint64_t>(d + 8), key_len = read_le<uint64_t>(d + 16);
        const uint64_t array_start = read_le<uint64_t>(d + 24);
        const uint64_t array_len = read_le<uint64_t>(d + 32);
        if (type >= KAS_NUM_TYPES || key_start != offset || key_len > size - key_start) {
            ret = TSG_ERR_FILE_FORMAT;
            break;
        }
        offset += key_len;
        tsg_kastore::Item it;
        it.type = type;
        it.key.assign((const char *) b + key_start, (size_t) key_len);
        it.array_start = array_start;
        it.array_len = array_len;
        k->items.push_back(std::move(it));
    }
    for (size_t j = 0; ret == 0 && j < k->items.size(); j++) {
        offset = (offset + 7) / 8 * 8;
        const auto &it = k->items[j];
        const uint64_t bytes = it.array_len * (uint64_t) type_size(it.type);
        if (it.array_start != offset || (it.array_len != 0 && bytes / it.array_len
                != (uint64_t) type_size(it.type)) || bytes > size - offset) {
            ret = TSG_ERR_FILE_FORMAT;
            break;
        }
        offset += bytes;
    }
    if (ret == 0 && offset != size) {
        ret = TSG_ERR_FILE_FORMAT;
    }
    if (ret != 0) {
        delete k;
        return ret;
    }
    *out = k;
    return 0;
}

int tsg_kastore_get(const tsg_kastore_t *k, const char *key, int32_t *type, int64_t *len,
    const void **data)
{
    for (const auto &it : k->items) {
        if (it.key == key) {
            *type = it.type;
            *len = (int64_t) it.array_len;
            *data = k->bytes.data() + it.array_start;
            return 0;
        }
    }
    return TSG_ERR_REQUIRED_COL_NOT_FOUND;
}

int tsg_kastore_free(tsg_kastore_t *k)
{
    delete k;
    return 0;
}

}  // extern "C"
