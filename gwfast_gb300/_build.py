"""Build the CUDA extension in-tree for sm_103a (nvcc, one translation unit per model, in parallel)."""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
INC = os.path.join(os.path.dirname(HERE), 'include')
OBJ = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libgwfast_gb300.so')
SOURCES = ('gwf_run_tf2.cu', 'gwf_run_phd.cu', 'gwf_run_phm.cu', 'gwf_run_tf2t.cu', 'gwf_run_nrt.cu', 'gwf_run_tf2e.cu',
           'gwf_run_tf2et.cu', 'gwf_run_nsbh.cu', 'gwf_cov.cu', 'gwf_api.cu', 'gwf_noalloc.cu', 'gwf_mixed.cu', 'gwf_mlp.cu')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-I' + CSRC, '-I' + INC]


def nvcc():
    exe = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(exe):
        raise RuntimeError('nvcc not found')
    return exe


def _stale(srcs):
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INC, 'gwfast_gb300.h'), __file__]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=()):
    """Compile csrc/*.cu and link libgwfast_gb300.so next to this file; returns its path."""
    if not force and not _stale(SOURCES):
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    exe = nvcc()
    procs = []
    for src in SOURCES:
        obj = os.path.join(OBJ, src.replace('.cu', '.o'))
        cmd = [exe] + ARCH + FLAGS + list(extra) + ['-c', os.path.join(CSRC, src), '-o', obj]
        if verbose:
            print(' '.join(cmd))
        procs.append((src, obj, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    objs = []
    errors = []
    for src, obj, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append('%s:\n%s' % (src, out))
        elif verbose and out.strip():
            print(out)
        objs.append(obj)
    if errors:
        raise RuntimeError('nvcc failed\n' + '\n'.join(errors))
    tmp = LIB + '.tmp'
    cmd = [exe] + ARCH + ['-shared', '-o', tmp] + objs + ['-lcudart']
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError('link failed\n' + r.stdout)
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(force='-f' in sys.argv, verbose='-v' in sys.argv))
