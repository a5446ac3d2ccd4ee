"""Headless hunt (bsf_worker hunt): the candidate log has the reference's
header and one row per exact-stage region, each row agreeing with the MEGA
record of the same region through the C ABI."""
import csv
import os
import subprocess

import numpy as np
import pytest

import betaseedfinder_gb300 as bsf

pytestmark = pytest.mark.gpu

HEADER = ("attempt,seed,stage0,stage0Y88,coarse,p20,upper,high,p19Pass,p19Score,p19Extreme,searchCenterChunkX,"
          "searchCenterChunkZ,matched,status,rawBlocks,verifiedBlocks,rawRadius,verifiedRadius,rawTouchesSide,"
          "verifiedTouchesSide,columns,width,depth,footprintArea,fillPercent,avgThickness,minY,maxY,centerX,centerZ,"
          "minX,maxX,minZ,maxZ,hotScanned,hotRadius,hotBlocks,hotTouchesSide,finalSource")


def test_hunt_writes_reference_candidate_rows(tmp_path):
    seq, worlds = 7_123_456_789, 16000
    regions = 8 * worlds - 3                        # the last world has 5 of its 8 centres
    # two batches of 8192 worlds: attempts continue across batches
    out = subprocess.run([bsf.WORKER_PATH, "hunt", str(seq), str(regions), "mega", "7", str(tmp_path), "8192"],
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    text = open(os.path.join(tmp_path, "hunter_candidates.csv")).read()
    assert text.splitlines()[0] == HEADER
    rows = list(csv.DictReader(text.splitlines()))
    seeds = np.array([bsf.splitmix_seed(seq, a) for a in range(1, worlds + 1)], dtype=np.int64)
    with bsf.Worker(capacity=worlds, profile="mega", centers=8, max_exact_radius=24) as w:
        _, recs = w.mega_search(seeds, radius=7)
    recs = [r for r in recs if r.world_index * 8 + r.center_index < regions]
    assert len(rows) == len(recs) > 0
    for row, r in zip(rows, recs):
        assert int(row["attempt"]) == r.world_index * 8 + r.center_index + 1
        assert int(row["seed"]) == r.seed
        assert (int(row["coarse"]), int(row["p20"]), int(row["upper"]), int(row["high"])) == \
               (r.coarse, r.p20, r.upper, r.high)
        assert int(row["stage0"]) == int(row["stage0Y88"]) == r.high
        assert row["p19Pass"] == "true"
        assert (int(row["searchCenterChunkX"]), int(row["searchCenterChunkZ"])) == (r.center_chunk_x, r.center_chunk_z)
        assert row["matched"] == ("true" if r.island.found else "false")
        if r.island.found:
            assert int(row["verifiedBlocks"]) == r.island.blocks and int(row["columns"]) == r.island.columns
            assert int(row["width"]) == r.island.max_x - r.island.min_x + 1
            assert row["status"].startswith("matched") or row["status"] == "duplicate_region_merged"
            assert row["finalSource"] in ("raw", "hot_scan", "duplicate_merged")
        else:
            assert row["status"] in ("no_match", "hot_scan_no_match") and row["finalSource"] == "none"
    manifest = open(os.path.join(tmp_path, "run_manifest.json")).read()
    assert '"seedsToCheck": %d' % regions in manifest and '"worldsChecked": %d' % worlds in manifest
    # manifest.txt as the app's run history reads it (RunRepository.parseManifest: split at the first '=',
    # trim both sides; RunRecord reads build/status/runLabel/epochs/checked/matches/topUpdates)
    lines = open(os.path.join(tmp_path, "manifest.txt")).read().splitlines()
    assert lines[0] == "BetaSeedFinder run manifest"
    kv = {}
    for line in lines:
        eq = line.find("=")
        if eq > 0:
            kv[line[:eq].strip()] = line[eq + 1:].strip()
    assert kv["status"] == "FINISHED" and int(kv["checked"]) == regions == int(kv["seedsToCheck"])
    assert int(kv["matches"]) == sum(1 for row in rows if row["matched"] == "true")
    assert 0 < int(kv["topUpdates"]) <= int(kv["matches"]) or int(kv["matches"]) == 0
    assert int(kv["startEpochMs"]) <= int(kv["endEpochMs"]) and float(kv["elapsedSeconds"]) >= 0
    assert kv["checkedUnit"] == "radius7Regions" and kv["gpuCoverageCentersPerWorld"] == "8"
    assert kv["huntProfileName"] == "MEGA 30k+" and kv["megaMode"] == "true"
    assert kv["deterministicSeedMode"] == "true" and int(kv["deterministicSeedSequenceSeed"]) == seq
    assert kv["chunkRadius"] == "7" and kv["minBlocks"] == "1000" and kv["minAvgThickness"] == "2.0"
    assert kv["effectiveP19MinScore"] == "4.02" and kv["hunterCoarseMinCells"] == "85"
    # the leaderboard holds the run's unique matches, best first (blocks, columns, area, thickness)
    unique = [row for row in rows if row["matched"] == "true"]
    want = sorted(((int(r["verifiedBlocks"]), int(r["columns"]), int(r["footprintArea"]),
                    int(r["verifiedBlocks"]) / max(1, int(r["columns"])), int(r["seed"])) for r in unique),
                  key=lambda t: t[:4], reverse=True)[:50]
    board = [row for row in csv.DictReader(open(os.path.join(tmp_path, "top_island_sideboards.csv")))
             if row["board"] == "largest"]
    assert [(int(b["seed"]), int(b["blocks"])) for b in board] == [(t[4], t[0]) for t in want]
    assert [int(b["rank"]) for b in board] == list(range(1, len(board) + 1))


def test_hunt_reject_audits_match_exact_scans(tmp_path):
    """Audited rejects (seed & mask == 0) get an exact scan; each audit row
    carries the region's stage outcome and the exact scan's island."""
    seq, worlds, mask = 99_001, 3000, 15
    out = subprocess.run([bsf.WORKER_PATH, "hunt", str(seq), str(8 * worlds), "mega", "5", str(tmp_path), "4096",
                          "1000", str(mask)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    text = open(os.path.join(tmp_path, "record_reject_audits.csv")).read()
    assert text.splitlines()[0] == (
        "attempt,seed,searchCenterChunkX,searchCenterChunkZ,rejectStage,rejectReason,p20,upper,high,p19Pass,"
        "p19Score,p19Extreme,coarse,exactScanMs,exactMatched,exactBlocks,exactColumns,exactWidth,exactDepth,"
        "exactMinY,exactMaxY,exactRadiusUsed,exactTouchesSideBorder")
    rows = list(csv.DictReader(text.splitlines()))
    assert len(rows) > 20
    seeds = np.array([bsf.splitmix_seed(seq, a) for a in range(1, worlds + 1)], dtype=np.int64)
    with bsf.Worker(capacity=worlds, profile="mega", centers=8, max_exact_radius=24) as w:
        w.mega_search(seeds, radius=5)
        regs = bsf.decode_records(w.last_region_records(worlds), 34)
        for row in rows[:40]:
            region = int(row["attempt"]) - 1
            seed = int(row["seed"])
            assert seed == seeds[region // 8] and seed & mask == 0
            assert int(row["p20"]) == regs["p20Counts"][region] and int(row["coarse"]) == regs["coarseScores"][region]
            assert int(row["rejectStage"]) in (1, 2, 4, 5, 6)
            isl = w.exact_scan(seed, int(row["searchCenterChunkX"]), int(row["searchCenterChunkZ"]), 5)
            assert row["exactMatched"] == ("true" if isl.found else "false")
            if isl.found:
                assert int(row["exactBlocks"]) == isl.blocks and int(row["exactMinY"]) == isl.min_y
