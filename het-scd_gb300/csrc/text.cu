// The text edge-list reader of `convert` (read_edges, src/convert.cpp:74-138)
// on the device.
//
// Semantics kept from the reference: lines end at '\n'; a line of more than
// 1023 characters makes the read fail (std::istream::getline into a 1024-byte
// buffer sets failbit; the reference still parses the first 1023 characters
// of that line, so a corrupt prefix is reported as a corrupt line); leading
// white space (isspace) is skipped; an empty line or one whose first
// non-blank character is '#' is ignored; otherwise two unsigned decimal
// numbers separated by white space must follow (unsigned wrap-around on
// overflow, anything after the second number ignored), else "line i is
// corrupt" with i counting every line from 1; the record is (min, max).  A
// NUL byte ends a line's content, as in the reference's C-string scan.  Only
// the first failing line matters: the reference stops there.
//
// Layout: the text is cut into 8 KB chunks; one pass counts the newlines of
// every chunk, a scan gives each chunk its first line number, a second pass
// writes every newline position; then one thread parses one line and a scan
// over the "is a record" flags places the records in file order.
#include "engine.cuh"

namespace scd {

namespace {

constexpr unsigned TPB = 256;
constexpr uint32_t CHUNK = 8192;   // bytes of text per block in the newline passes
constexpr uint32_t MAX_LINE = 1023;

__global__ void __launch_bounds__(TPB)
k_count_newlines(const char *__restrict__ text, uint64_t bytes, uint32_t *per_chunk) {
    __shared__ uint32_t ws[TPB / 32];
    const uint64_t c0 = (uint64_t)blockIdx.x * CHUNK;
    uint32_t k = 0;
    for (uint64_t i = c0 + threadIdx.x; i < bytes && i < c0 + CHUNK; i += TPB) k += text[i] == '\n';
    k = warp_sum(k);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = k;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < TPB / 32; w++) t += ws[w];
        per_chunk[blockIdx.x] = t;
    }
}

// newline positions in text order: chunk c writes its newlines from nl_off[c]
__global__ void __launch_bounds__(TPB)
k_newline_positions(const char *__restrict__ text, uint64_t bytes, const uint32_t *__restrict__ nl_off,
                    uint64_t *nl_pos) {
    __shared__ uint32_t ws[TPB / 32];
    __shared__ uint32_t base;
    const uint64_t c0 = (uint64_t)blockIdx.x * CHUNK;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) base = nl_off[blockIdx.x];
    __syncthreads();
    for (uint64_t r0 = c0; r0 < bytes && r0 < c0 + CHUNK; r0 += TPB) {
        const uint64_t i = r0 + threadIdx.x;
        const bool nl = i < bytes && i < c0 + CHUNK && text[i] == '\n';
        const unsigned b = __ballot_sync(FULL, nl);
        if (lane == 0) ws[w] = __popc(b);
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (int k = 0; k < TPB / 32; k++) {
            before += k < w ? ws[k] : 0u;
            total += ws[k];
        }
        if (nl) nl_pos[base + before + __popc(b & lanemask_lt())] = i;
        __syncthreads();
        if (threadIdx.x == 0) base += total;
        __syncthreads();
    }
}

__device__ __forceinline__ bool is_space(char ch) {
    return ch == ' ' || ch == '\t' || ch == '\n' || ch == '\v' || ch == '\f' || ch == '\r';
}
__device__ __forceinline__ bool is_digit(char ch) { return ch >= '0' && ch <= '9'; }

// status per line: 0 ignored, 1 record, 2 corrupt, 3 read failure (line too long)
__global__ void k_parse_lines(const char *__restrict__ text, uint64_t bytes, const uint64_t *__restrict__ nl_pos,
                              uint32_t lines, uint8_t *status, uint32_t *rec, unsigned long long *first_error) {
    for (uint32_t L = blockIdx.x * blockDim.x + threadIdx.x; L < lines; L += gridDim.x * blockDim.x) {
        const uint64_t beg = L == 0 ? 0 : nl_pos[L - 1] + 1;
        const uint64_t end = L + 1 < lines ? nl_pos[L] : bytes;
        const uint64_t len = end - beg;
        // the reference's buffer holds the first 1023 characters of the line
        const uint64_t stop = beg + (len > MAX_LINE ? MAX_LINE : len);
        uint64_t k = beg;
        auto at = [&](uint64_t q) -> char { return q < stop ? text[q] : '\0'; };
        uint8_t st = 1;
        uint32_t a = 0, b = 0;
        while (is_space(at(k))) k++;
        char ch = at(k);
        if (ch == '\0' || ch == '#') {
            st = 0;
        } else if (!is_digit(ch)) {
            st = 2;
        } else {
            while (is_digit(at(k))) a = 10u * a + (uint32_t)(at(k++) - '0');
            while (is_space(at(k))) k++;
            if (!is_digit(at(k))) st = 2;
            else
                while (is_digit(at(k))) b = 10u * b + (uint32_t)(at(k++) - '0');
        }
        if (st != 2 && len > MAX_LINE) st = 3;   // parsed, then the failed read stops the input
        status[L] = st;
        rec[2 * (uint64_t)L] = a < b ? a : b;
        rec[2 * (uint64_t)L + 1] = a < b ? b : a;
        if (st >= 2) atomicMin(first_error, ((unsigned long long)L << 2) | st);
    }
}

struct IsRecord {
    const uint8_t *status;
    __device__ uint32_t operator[](size_t i) const { return status[i] == 1; }
};

__global__ void k_compact_records(const uint8_t *__restrict__ status, const uint32_t *__restrict__ rec,
                                  const uint32_t *__restrict__ pos, uint32_t lines, uint32_t *pairs) {
    for (uint32_t L = blockIdx.x * blockDim.x + threadIdx.x; L < lines; L += gridDim.x * blockDim.x)
        if (status[L] == 1) {
            pairs[2 * (uint64_t)pos[L]] = rec[2 * (uint64_t)L];
            pairs[2 * (uint64_t)pos[L] + 1] = rec[2 * (uint64_t)L + 1];
        }
}

}  // namespace

// Parses text (device memory) into (min, max) records in file order; returns
// their number and leaves them in out.  Throws SCD_ERR_FORMAT as the reference
// reports the first failing line.
uint64_t parse_edge_text(Ctx &c, const char *text, uint64_t bytes, DevBuf<uint32_t> &out) {
    cudaStream_t s = c.stream;
    const uint64_t chunks = (bytes + CHUNK - 1) / CHUNK;
    if (chunks >= (1ull << 31)) throw Error(SCD_ERR_LIMIT, "text larger than 2^31 chunks");
    DevBuf<uint32_t> per((size_t)chunks + 1, s), nl_off((size_t)chunks + 1, s);
    uint32_t nl = 0;
    if (chunks) {
        k_count_newlines<<<(unsigned)chunks, TPB, 0, s>>>(text, bytes, per.get());
        CK_LAUNCH("k_count_newlines");
        scan_exclusive<uint32_t>((const uint32_t *)per.get(), nl_off.get(), chunks, s);
        CK(cudaMemcpyAsync(&nl, nl_off.get() + chunks, 4, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    if (nl >= 0xfffffffeu) throw Error(SCD_ERR_LIMIT, "more than 2^32-2 text lines");
    const uint32_t lines = nl + 1;   // the piece after the last newline (possibly empty) is a line too
    DevBuf<uint64_t> nl_pos(nl ? nl : 1, s);
    if (chunks && nl) {
        k_newline_positions<<<(unsigned)chunks, TPB, 0, s>>>(text, bytes, nl_off.get(), nl_pos.get());
        CK_LAUNCH("k_newline_positions");
    }
    DevBuf<uint8_t> status(lines, s);
    DevBuf<uint32_t> rec(2 * (size_t)lines, s), pos((size_t)lines + 1, s);
    DevBuf<unsigned long long> err(1, s);
    CK(cudaMemsetAsync(err.get(), 0xff, 8, s));
    k_parse_lines<<<grid_for(lines, TPB), TPB, 0, s>>>(text, bytes, nl_pos.get(), lines, status.get(), rec.get(),
                                                       err.get());
    CK_LAUNCH("k_parse_lines");
    scan_exclusive<uint32_t>(IsRecord{status.get()}, pos.get(), lines, s);
    unsigned long long e = 0;
    uint32_t count = 0;
    CK(cudaMemcpyAsync(&e, err.get(), 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&count, pos.get() + lines, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    c.launches += 4;
    if (e != ~0ull) {
        const uint64_t line = (e >> 2) + 1;
        if ((e & 3) == 2) throw Error(SCD_ERR_FORMAT, "line " + std::to_string(line) + " is corrupt");
        throw Error(SCD_ERR_FORMAT, "an error occured while reading input file (line " + std::to_string(line) +
                                        " is longer than 1023 characters)");
    }
    out.alloc(2 * (size_t)count + 2, s);
    k_compact_records<<<grid_for(lines, TPB), TPB, 0, s>>>(status.get(), rec.get(), pos.get(), lines, out.get());
    CK_LAUNCH("k_compact_records");
    c.launches++;
    return count;
}

}  // namespace scd
