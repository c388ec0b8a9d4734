// XLA FFI handlers over the C ABI: the custom-call targets an FRX/JAX program
// registers with frx.ffi.register_ffi_target and calls with frx.ffi.ffi_call,
// the seam the reference uses for its host-FS hop (zorch/transcript.py:
// 1005-1035 registration, 1098-1100 the call). Each handler takes XLA's
// buffers and stream, forwards them to the zc_* entry point and maps a status
// to an FFI error; it holds no state between calls (the transcript state
// crosses in and out as buffers, as the reference's FFI contract requires,
// zorch/transcript.py:1015-1021).
//
// Built into libzc_xla.so only where the XLA FFI headers are present
// (zorch_gb300/build.py: XLA_FFI_INCLUDE_DIR or an installed jaxlib's include
// directory); the library then links against libzc.so.
//
// Field data are the Montgomery u32 words of zk_dtypes' *_mont dtypes, passed
// as U32 buffers (a caller views babybear_mont / koalabear_mont arrays as
// uint32 on the way in and back on the way out).
#include <cuda_runtime.h>
#include <stdint.h>

#include "xla/ffi/api/ffi.h"
#include "zc.h"

namespace ffi = xla::ffi;

namespace {

ffi::Error status_error(zc_status s) {
  if (s == ZC_OK) return ffi::Error::Success();
  const ffi::ErrorCode code = (s == ZC_BAD_SHAPE || s == ZC_NOT_POW2 || s == ZC_BAD_ARG)
                                  ? ffi::ErrorCode::kInvalidArgument
                              : s == ZC_UNSUPPORTED ? ffi::ErrorCode::kUnimplemented
                              : s == ZC_OOM         ? ffi::ErrorCode::kResourceExhausted
                                                    : ffi::ErrorCode::kInternal;
  return ffi::Error(code, zc_last_error());
}

int log2_exact(int64_t x) {
  int l = 0;
  while (((int64_t)1 << l) < x) l++;
  return ((int64_t)1 << l) == x ? l : -1;
}

zc_field field_of(int64_t f) { return f == 1 ? ZC_FIELD_KOALABEAR : ZC_FIELD_BABYBEAR; }

// ReedSolomon.encode (zorch/coding/reed_solomon.py:177-188) -> zc_rs_encode.
// coeffs [..., k]; out [..., k << log_blowup]; ws: the workspace, sized by the
// caller with zc_rs_encode_workspace_bytes (an extra result, so XLA allocates
// it from its own pool).
ffi::Error RsEncode(cudaStream_t stream, ffi::Buffer<ffi::U32> coeffs,
                    ffi::ResultBuffer<ffi::U32> out, ffi::ResultBuffer<ffi::U8> ws, int64_t field,
                    int64_t log_blowup, int64_t shift_mont, int64_t bit_reversed) {
  const auto dims = coeffs.dimensions();
  if (dims.size() < 1) return status_error(ZC_BAD_SHAPE);
  const int64_t k = dims.back();
  const int log_k = log2_exact(k);
  if (log_k < 0) return status_error(ZC_NOT_POW2);
  const int64_t batch = (int64_t)coeffs.element_count() / k;
  auto fn = bit_reversed ? zc_rs_encode_bitrev : zc_rs_encode;
  return status_error(fn(field_of(field), coeffs.typed_data(), batch, log_k, (int)log_blowup,
                         (uint32_t)shift_mont, 0, out->typed_data(), ws->untyped_data(),
                         ws->size_bytes(), stream));
}

// MerkleTree.commit over pair leaves or row leaves (zorch/commit/merkle.py:
// 118-202) -> zc_merkle_commit. leaves: the codeword [w, n] (column-major
// rows, leaf r = column r) when pair = 0, or one [n] codeword whose pair
// leaves (cw[p], cw[p + n/2]) are committed when pair = 1; layers: the
// (2L - 1) x 8 digest words. A built-in BabyBear instance hashes (the handle
// is created on first use).
ffi::Error MerkleCommit(cudaStream_t stream, ffi::Buffer<ffi::U32> leaves,
                        ffi::ResultBuffer<ffi::U32> layers, int64_t pair) {
  const auto dims = leaves.dimensions();
  if (dims.size() < 1) return status_error(ZC_BAD_SHAPE);
  const zc_poseidon2* p = nullptr;
  zc_status s = zc_poseidon2_builtin(ZC_FIELD_BABYBEAR, &p);
  if (s != ZC_OK) return status_error(s);
  const int64_t n = dims.back();
  const int64_t w = (int64_t)leaves.element_count() / n;
  zc_leaves lv;
  lv.base = leaves.typed_data();
  if (pair) {
    lv.num_leaves = n / 2;
    lv.groups = 2;
    lv.group_len = 1;
    lv.group_stride = n / 2;
  } else {
    lv.num_leaves = n;
    lv.groups = (int32_t)w;
    lv.group_len = 1;
    lv.group_stride = n;
  }
  return status_error(zc_merkle_commit(p, lv, layers->typed_data(), stream));
}

// PreFoldPairCommitRound's fold of round r fused with the commit of round
// r + 1 (zorch/pcs/fold.py:90-115) -> zc_fri_fold_commit. cw: [n] base or
// [n, 4] EF4 layer; beta: 1 or 4 words; folded: the next layer; layers: its
// pair-leaf tree (n/4 leaves).
ffi::Error FriFoldCommit(cudaStream_t stream, ffi::Buffer<ffi::U32> cw,
                         ffi::Buffer<ffi::U32> beta, ffi::ResultBuffer<ffi::U32> folded,
                         ffi::ResultBuffer<ffi::U32> layers, int64_t shift_mont) {
  const zc_poseidon2* p = nullptr;
  zc_status s = zc_poseidon2_builtin(ZC_FIELD_BABYBEAR, &p);
  if (s != ZC_OK) return status_error(s);
  const auto dims = cw.dimensions();
  if (dims.size() < 1) return status_error(ZC_BAD_SHAPE);
  const int ef_in = dims.size() == 2 && dims[1] == 4;
  const int64_t n = dims[0];
  const int ef_beta = beta.element_count() == 4;
  return status_error(zc_fri_fold_commit(p, cw.typed_data(), n, ef_in, beta.typed_data(), ef_beta,
                                         (uint32_t)shift_mont, 0, folded->typed_data(),
                                         layers->typed_data(), stream));
}

// The six-operand Fiat-Shamir hop (zorch/transcript.py:1015-1021, 1056-1112)
// on the device -> zc_duplex_hop: the five state operands and the values in,
// the five advanced operands and `n` challenge words out.
ffi::Error DuplexHop(cudaStream_t stream, ffi::Buffer<ffi::U32> in_buf,
                     ffi::Buffer<ffi::U32> out_buf, ffi::Buffer<ffi::U32> sponge,
                     ffi::Buffer<ffi::U32> in_pos, ffi::Buffer<ffi::U32> out_pos,
                     ffi::Buffer<ffi::U32> values, ffi::ResultBuffer<ffi::U32> in_buf_o,
                     ffi::ResultBuffer<ffi::U32> out_buf_o, ffi::ResultBuffer<ffi::U32> sponge_o,
                     ffi::ResultBuffer<ffi::U32> in_pos_o, ffi::ResultBuffer<ffi::U32> out_pos_o,
                     ffi::ResultBuffer<ffi::U32> challenges) {
  const zc_poseidon2* p = nullptr;
  zc_status s = zc_poseidon2_builtin(ZC_FIELD_BABYBEAR, &p);
  if (s != ZC_OK) return status_error(s);
  return status_error(zc_duplex_hop(
      p, in_buf.typed_data(), out_buf.typed_data(), sponge.typed_data(), in_pos.typed_data(),
      out_pos.typed_data(), values.typed_data(), (int64_t)values.element_count(),
      (int32_t)challenges->element_count(), in_buf_o->typed_data(), out_buf_o->typed_data(),
      sponge_o->typed_data(), in_pos_o->typed_data(), out_pos_o->typed_data(),
      challenges->typed_data(), stream));
}

}  // namespace

XLA_FFI_DEFINE_HANDLER_SYMBOL(zc_rs_encode_ffi, RsEncode,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::U32>>()
                                  .Ret<ffi::Buffer<ffi::U32>>()
                                  .Ret<ffi::Buffer<ffi::U8>>()
                                  .Attr<int64_t>("field")
                                  .Attr<int64_t>("log_blowup")
                                  .Attr<int64_t>("shift_mont")
                                  .Attr<int64_t>("bit_reversed"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(zc_merkle_commit_ffi, MerkleCommit,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::U32>>()
                                  .Ret<ffi::Buffer<ffi::U32>>()
                                  .Attr<int64_t>("pair"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(zc_fri_fold_commit_ffi, FriFoldCommit,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::U32>>()
                                  .Arg<ffi::Buffer<ffi::U32>>()
                                  .Ret<ffi::Buffer<ffi::U32>>()
                                  .Ret<ffi::Buffer<ffi::U32>>()
                                  .Attr<int64_t>("shift_mont"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(zc_duplex_hop_ffi, DuplexHop,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::U32>>()
                                  .Arg<ffi::Buffer<ffi::U32>>()
                                  .Arg<ffi::Buffer<ffi::U32>>()
                                  .Arg<ffi::Buffer<ffi::U32>>()
                                  .Arg<ffi::Buffer<ffi::U32>>()
                                  .Arg<ffi::Buffer<ffi::U32>>()
                                  .Ret<ffi::Buffer<ffi::U32>>()
                                  .Ret<ffi::Buffer<ffi::U32>>()
                                  .Ret<ffi::Buffer<ffi::U32>>()
                                  .Ret<ffi::Buffer<ffi::U32>>()
                                  .Ret<ffi::Buffer<ffi::U32>>()
                                  .Ret<ffi::Buffer<ffi::U32>>());
