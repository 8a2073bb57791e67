#!/bin/sh
# Writes the b200 program stdout captures of this directory.  Run on a
# machine with an sm_103 GPU after the build (__graft_entry__.build()), from
# the repository root.  PROFILING_FNAME makes the programs print the
# "<kernel> regcount" and per-sweep "<kernel> kernel time" lines the suite's
# benchmark harness parses for GPU targets.
set -e
BIN=kernelgen-perf-tests_gb300/build/bin
OUT=tests/golden
PROFILING_FNAME=laplacian $BIN/laplacian_b200 512 256 256 10 > $OUT/b200_stdout_laplacian_512x256x256x10.txt
PROFILING_FNAME=gameoflife $BIN/gameoflife_b200 512 65536 10 > $OUT/b200_stdout_gameoflife_512x65536x10.txt
PROFILING_FNAME=tricubic2 B200_MODE=graph $BIN/tricubic2_b200 512 256 256 10 > $OUT/b200_stdout_tricubic2_graph_512x256x256x10.txt
