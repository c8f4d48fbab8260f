"""`python -m verion_gb300.exr_diff reference.exr test.exr [more.exr ...]`: the reference's
`exr_diff` (crates/verion-render-io/examples/exr_diff.rs): compares the Beauty of each test image
with the reference's; gates worst channel mean within 1% and worst 4x4 block mean within 2%
(`EXR_DIFF_CHANNEL` / `EXR_DIFF_BLOCK` replace them), reports MAE over the mean and PSNR. Prints
PASS / FAIL per image; exits 1 when any fails, 2 on unreadable or mismatched files."""
import os
import sys

from .exr import beauty_rec709, diff, read_exr


def main(argv=None) -> int:
    args = list(sys.argv[1:] if argv is None else argv)
    if len(args) < 2:
        print("usage: exr_diff reference.exr test.exr [more.exr ...]", file=sys.stderr)
        return 2
    gc = float(os.environ.get("EXR_DIFF_CHANNEL", "0.01"))
    gb = float(os.environ.get("EXR_DIFF_BLOCK", "0.02"))

    def load(p):
        try:
            img = read_exr(p)
        except (OSError, ValueError, KeyError) as e:
            print(f"{p}: {e}", file=sys.stderr)
            sys.exit(2)
        return img.width, img.height, beauty_rec709(img)

    w, h, r = load(args[0])
    ok = True
    for path in args[1:]:
        tw, th, t = load(path)
        if (tw, th) != (w, h):
            print(f"{path}: size {tw}x{th} differs from {w}x{h}", file=sys.stderr)
            return 2
        d = diff(r, t, w, h, gc, gb)
        ok &= d["pass"]
        print(f"{path}: channel {d['channel'] * 100:.2f}% block {d['block'] * 100:.2f}% "
              f"mae/mean {d['mae_over_mean']:.4f} psnr {d['psnr_db']:.1f} dB {'PASS' if d['pass'] else 'FAIL'}")
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
