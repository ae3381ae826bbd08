import os
import subprocess
import sys

from autopdex_gb300 import build as B

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    src = os.path.join(HERE, "throughput_probe.cu")
    exe = os.path.join(B.LIBDIR, "throughput_probe")
    os.makedirs(B.LIBDIR, exist_ok=True)
    subprocess.run([B._nvcc()] + B.ARCH + ["-O3", "-o", exe, src], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    sys.stdout.write(r.stdout)
    sys.exit(r.returncode)


if __name__ == "__main__":
    main()
