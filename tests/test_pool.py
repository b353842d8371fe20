"""The batch's device memory pool (csrc/hc_pool.h), exercised on the host.

The pool's arena source is a template parameter; this test compiles the
header with g++ against a backend that hands out host memory and can be told
to refuse, then checks first-fit reuse, alignment, merging of freed
neighbours, the exact-size fallback when a whole arena does not fit, and
trim() returning wholly free arenas.
"""
import os
import subprocess
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "hydro-cl-lua_gb300", "csrc")
CUDA_INC = "/usr/local/cuda/include"

PROGRAM = textwrap.dedent(r"""
    #include "hc_pool.h"
    #include <cstdio>
    #include <cstdlib>
    #include <cstdint>

    static size_t g_limit = (size_t)1 << 40;   // bytes the fake device still has
    static size_t g_live = 0, g_calls = 0;
    struct FakeArenas {
        static cudaError_t alloc(void** p, size_t b) {
            ++g_calls;
            if (b > g_limit) return cudaErrorMemoryAllocation;
            *p = std::aligned_alloc(4096, (b + 4095) / 4096 * 4096);
            g_limit -= b; g_live += b;
            return cudaSuccess;
        }
        static void free(void* p) { std::free(p); }
        static void clear_error() {}
    };
    #define CHECK(c) do { if (!(c)) { std::printf("FAIL line %d: %s\n", __LINE__, #c); return 1; } } while (0)

    int main() {
        {
            hc::DevicePoolT<FakeArenas> pool(1 << 20);
            void *a, *b, *c, *d;
            CHECK(pool.alloc(1000, &a) == cudaSuccess);
            CHECK(pool.alloc(3000, &b) == cudaSuccess);
            CHECK(pool.alloc(5000, &c) == cudaSuccess);
            CHECK(pool.num_arenas() == 1);
            CHECK(((uintptr_t)a % 256) == 0 && ((uintptr_t)b % 256) == 0 && ((uintptr_t)c % 256) == 0);
            CHECK((char*)b - (char*)a == 1024);          // 1000 rounded to 256
            CHECK((char*)c - (char*)b == 3072);
            // free the middle one: first fit reuses it for a request that fits
            pool.release(b, 3000);
            CHECK(pool.alloc(2048, &d) == cudaSuccess && d == b);
            pool.release(d, 2048);
            // freeing a and the hole next to it merges them into one range
            pool.release(a, 1000);
            CHECK(pool.alloc(4096, &d) == cudaSuccess && d == a);
            pool.release(d, 4096);
            pool.release(c, 5000);
            CHECK(pool.free_bytes() == (size_t)1 << 20);    // everything merged back
            // bigger than an arena: an arena of its own
            CHECK(pool.alloc((size_t)3 << 20, &d) == cudaSuccess);
            CHECK(pool.num_arenas() == 2);
            pool.release(d, (size_t)3 << 20);
            CHECK(pool.trim() == ((size_t)1 << 20) + ((size_t)3 << 20));
            CHECK(pool.num_arenas() == 0 && pool.reserved() == 0);
        }
        {
            // the device has room for 1.5 arenas: the second request gets an
            // exact-size arena; once that is used up, trim() frees idle arenas
            g_limit = (size_t)3 << 19;
            hc::DevicePoolT<FakeArenas> pool(1 << 20);
            void *a, *b, *c;
            CHECK(pool.alloc(1 << 20, &a) == cudaSuccess);
            CHECK(pool.alloc(1 << 18, &b) == cudaSuccess);
            CHECK(pool.num_arenas() == 2 && pool.reserved() == ((size_t)1 << 20) + ((size_t)1 << 18));
            CHECK(pool.alloc(1 << 19, &c) != cudaSuccess);  // nothing idle to trim
            pool.release(a, 1 << 20);
            CHECK(pool.alloc(1 << 19, &c) == cudaSuccess);  // reuses the idle arena, no new one
            CHECK(pool.num_arenas() == 2);
        }
        std::printf("OK\n");
        return 0;
    }
""")


def test_device_pool_host(tmp_path):
    if not os.path.isdir(CUDA_INC):
        pytest.skip("CUDA headers not installed")
    src = tmp_path / "pool_test.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "pool_test"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", CSRC, "-I", CUDA_INC, str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stdout + r.stderr
