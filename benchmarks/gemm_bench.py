"""Throughput of the library's GEMMs (FP64 and emulated FP64) on one GPU.

  python -m benchmarks.gemm_bench M N K [--prec emu|fp64] [--slices S] [--reps R] [--cublas]

Operands are random FP64 device buffers (column-major); timing uses CUDA
events on the library stream after one warm-up launch.
"""
import argparse
import json


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("M", type=int)
    ap.add_argument("N", type=int)
    ap.add_argument("K", type=int)
    ap.add_argument("--prec", default="emu", choices=["emu", "fp64"])
    ap.add_argument("--slices", type=int, default=6)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--cublas", action="store_true",
                    help="with --prec fp64, also time cuBLAS DGEMM on the same shape")
    args = ap.parse_args()
    import torch
    from sisi4s_gb300 import capi
    ctx = capi.Context(0)
    ctx.set_emulation(args.slices, 0.0)
    M, N, K = args.M, args.N, args.K
    a = torch.randn(M * K, dtype=torch.float64, device="cuda")
    b = torch.randn(K * N, dtype=torch.float64, device="cuda")
    c = torch.zeros(M * N, dtype=torch.float64, device="cuda")
    prec = capi.PREC_EMU if args.prec == "emu" else capi.PREC_FP64
    torch.cuda.synchronize()

    def run():
        ctx.check(ctx.lib.gbcc_dgemm(ctx.h, 0, 0, M, N, K, 1.0, a.data_ptr(), M,
                                     b.data_ptr(), K, 0.0, c.data_ptr(), M, prec))
    run()
    stream = torch.cuda.ExternalStream(ctx.stream)
    torch.cuda.synchronize()
    ctx.profile(True)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.reps):
        run()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.reps
    st = ctx.gemm_stats()
    out = {"M": M, "N": N, "K": K, "prec": args.prec, "slices": args.slices,
           "ms_per_gemm": ms, "fp64_equiv_tflops": 2.0 * M * N * K / ms / 1e9}
    if st["launches"]:
        out["tensor_kernel_ms"] = st["ms"] / st["launches"]
        out["tensor_kernel_bf16_tflops"] = st["tc_flops"] / st["ms"] / 1e9
    if args.cublas and args.prec == "fp64":
        # the library DGEMM of the same shape (cuBLAS through torch), as the
        # FP64 reference point of this GPU
        A = a.view(K, M).t()
        B = b.view(N, K).t()
        torch.matmul(A, B)
        torch.cuda.synchronize()
        c0 = torch.cuda.Event(enable_timing=True)
        c1 = torch.cuda.Event(enable_timing=True)
        c0.record()
        for _ in range(args.reps):
            torch.matmul(A, B)
        c1.record()
        torch.cuda.synchronize()
        cms = c0.elapsed_time(c1) / args.reps
        out.update(cublas_ms=cms, cublas_tflops=2.0 * M * N * K / cms / 1e9)
    print(json.dumps(out))
    ctx.close()


if __name__ == "__main__":
    main()
