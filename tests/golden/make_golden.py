"""Write tests/golden/reference_known_answers.json.

The known answers below are the expected values that PointNeighbors.jl's own test suite
asserts for the GridNeighborhoodSearch / FullGridCellList path (file:line cited per case).
Julia is not available here, so the reference cannot be executed; its tests were read as
text and their inputs and expected outputs are restated as data.  Point indices in the
JSON are the reference's 1-based indices; coordinates are given point by point (the
columns of the reference's `T[d, N]` matrices).

Run:  python tests/golden/make_golden.py
"""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def lattice(rng_vals, ndims):
    """Iterators.product(range, range[, range]) collected column by column: first index
    fastest (test/nhs_grid.jl:93,158)."""
    n = len(rng_vals)
    pts = []
    if ndims == 2:
        for j in range(n):
            for i in range(n):
                pts.append([rng_vals[i], rng_vals[j]])
    else:
        for k in range(n):
            for j in range(n):
                for i in range(n):
                    pts.append([rng_vals[i], rng_vals[j], rng_vals[k]])
    return pts


def main():
    # collect(-0.25:0.1:0.35): Julia's float ranges give the correctly rounded decimals.
    rng = [-0.25, -0.15, -0.05, 0.05, 0.15, 0.25, 0.35]
    cases = {}

    # test/nhs_grid.jl:62-86 -- saturating cell coordinates at the limits.
    t63 = 9223372036854775807
    cases["cell_coords_limits"] = {
        "source": "test/nhs_grid.jl:62-86",
        "radius": 1.0,
        "coords": [["inf", "-inf"], ["nan", 0.0], [float(t63) + 1.0, -float(t63) - 1.0]],
        # DictionaryCellList: floor_to_int(x / r)
        "dict_expected": [[t63, -t63 - 1], [t63, 0], [t63, -t63 - 1]],
        # FullGridCellList(min=(0,0), max=(1,1), r=1): (..) .+ 1 with Int64 wrap-around
        "full_grid": {"min_corner": [0.0, 0.0], "max_corner": [1.0, 1.0]},
        "full_expected": [[-t63 - 1, -t63], [-t63 - 1, 2], [-t63 - 1, -t63]],
    }

    # test/nhs_grid.jl:88-151 -- 2D candidate lists (DictionaryCellList).
    p2 = lattice(rng, 2)
    cases["rect_2d"] = {
        "source": "test/nhs_grid.jl:88-151",
        "coords": p2,
        "checks": [
            {"radius": 0.1, "shift": [0.0, 0.0], "query": [0.05, 0.05],
             "expected": [17, 18, 19, 24, 25, 26, 31, 32, 33]},
            {"radius": 0.1, "shift": [1.4, -3.5], "query": [0.05, 0.05], "expected": []},
            {"radius": 0.1, "shift": [1.4, -3.5], "query_shifted": True,
             "query": [0.05, 0.05], "expected": [17, 18, 19, 24, 25, 26, 31, 32, 33]},
            {"radius": 0.2, "shift": [0.0, 0.0], "query": [0.05, 0.05],
             "expected": [9, 10, 11, 12, 13, 14, 16, 17, 18, 19, 20, 21, 23, 24, 25, 26, 27,
                          28, 30, 31, 32, 33, 34, 35, 37, 38, 39, 40, 41, 42, 44, 45, 46, 47,
                          48, 49]},
            {"radius": 0.2, "shift": [0.4, -0.4], "query": [0.05, 0.05],
             "expected": [36, 37, 38, 43, 44, 45]},
        ],
    }

    # test/nhs_grid.jl:153-196 -- 3D candidate lists (DictionaryCellList).
    p3 = lattice(rng, 3)
    l3 = [115, 116, 117, 122, 123, 124, 129, 130, 131, 164, 165, 166, 171, 172, 173, 178,
          179, 180, 213, 214, 215, 220, 221, 222, 227, 228, 229]
    cases["rect_3d"] = {
        "source": "test/nhs_grid.jl:153-196",
        "coords": p3,
        "checks": [
            {"radius": 0.1, "shift": [0.0, 0.0, 0.0], "query": [0.05, 0.05, 0.05],
             "expected": l3},
            {"radius": 0.1, "shift": [1.4, -3.5, 0.8], "query": [0.05, 0.05, 0.05],
             "expected": []},
            {"radius": 0.1, "shift": [1.4, -3.5, 0.8], "query_shifted": True,
             "query": [0.05, 0.05, 0.05], "expected": l3},
        ],
    }

    # test/nhs_grid.jl:197-225 -- FullGridCellList, update! with eachindex_y = 120:220.
    cases["eachindex_y_3d"] = {
        "source": "test/nhs_grid.jl:197-225",
        "coords": p3,
        "radius": 0.1,
        "shift": [1.4, -3.5, 0.8],
        "eachindex_y": [120, 220],
        "query1": [0.05, 0.05, 0.05],
        "expected1": [],
        "query2_shifted": True,
        "expected2": [122, 123, 124, 129, 130, 131, 164, 165, 166, 171, 172, 173, 178, 179,
                      180, 213, 214, 215, 220],
    }

    # test/nhs_grid.jl:228-292 (candidates) and test/neighborhood_search.jl:59-184
    # (neighbours) -- periodic boxes, r = 0.1.
    base2 = [[-0.08, -0.12], [0.0, -0.05], [0.18, -0.09], [0.1, 0.15], [-0.08, 0.39]]
    base2b = [[-0.08, -0.12], [0.0, -0.05], [0.18, -0.09], [0.1, 0.15], [-0.08, 0.42]]
    base3 = [[-0.08, -0.12, 0.14], [0.0, -0.05, 0.34], [0.18, -0.09, 0.12],
             [0.1, 0.15, 0.06], [-0.08, 0.39, 0.13]]
    cases["periodic_candidates"] = {
        "source": "test/nhs_grid.jl:228-292",
        "radius": 0.1,
        "setups": [
            {"name": "Simple Example 2D", "coords": base2,
             "box_min": [-0.1, -0.2], "box_max": [0.2, 0.4]},
            {"name": "Box Not Multiple of Search Radius 2D", "coords": base2b,
             "offset": [0.0017, 0.005],
             "box_min": [-0.1, -0.2], "box_max": [0.205, 0.43]},
            {"name": "Simple Example 3D", "coords": base3,
             "box_min": [-0.1, -0.2, 0.05], "box_max": [0.2, 0.4, 0.35]},
        ],
        "expected": [[1, 2, 3, 5], [1, 2, 3], [1, 2, 3], [4], [1, 5]],
    }
    cases["periodic_neighbors"] = {
        "source": "test/neighborhood_search.jl:59-184",
        "radius": 0.1,
        "setups": [
            {"name": "Simple Example 2D", "coords": base2,
             "box_min": [-0.1, -0.2], "box_max": [0.2, 0.4]},
            {"name": "Box Not Multiple of Search Radius 2D", "coords": base2b,
             "box_min": [-0.1, -0.2], "box_max": [0.205, 0.43]},
            {"name": "Simple Example 3D", "coords": base3,
             "box_min": [-0.1, -0.2, 0.05], "box_max": [0.2, 0.4, 0.35]},
        ],
        "expected": [[1, 3, 5], [2], [1, 3], [4], [1, 5]],
    }

    # test/nhs_grid.jl:294-325 -- split-cell regression (DictionaryCellList, periodic).
    cases["split_cells"] = {
        "source": "test/nhs_grid.jl:294-325",
        "radius": 1.0,
        "coords": [[-1.4, 0.0], [1.9, 0.0]],
        "box_min": [-1.5, 0.0], "box_max": [2.5, 3.0],
        "expected": [[1, 2], [1, 2]],
    }

    # test/neighborhood_search.jl:4-57 -- rounding at periodic edges (Float32 and Float64).
    cases["periodic_rounding"] = {
        "source": "test/neighborhood_search.jl:4-57",
        "box_min": [0.0, 0.0], "box_max": [1.0, 1.0], "radius": 0.1,
        # "prev"/"next" mean prevfloat/nextfloat of the given value in T
        "coords": [[["prev", 0.0], 0.5], [0.0, 0.5], [["next", 0.0], 0.5],
                   [["prev", 1.0], 0.5], [1.0, 0.5], [["next", 1.0], 0.5],
                   [0.5, ["prev", 0.0]], [0.5, 0.0], [0.5, ["next", 0.0]],
                   [0.5, ["prev", 1.0]], [0.5, 1.0], [0.5, ["next", 1.0]]],
    }

    # test/cell_lists/full_grid.jl:18-66 -- padded corners and out-of-domain errors.
    cases["full_grid_bounds"] = {
        "source": "test/cell_lists/full_grid.jl:18-66",
        "min_corner": 0.0, "max_corner": 10.0, "radius": 1.0,
        "expected_min_pad": -1.001, "expected_max_pad": 10.0 + 1.001,
        # value placed at y[1, 7] (first coordinate of point 7) and whether it must fail
        "initialize": [["nan", True], [-0.01, True], [11.01, True], [0.0, False]],
        "update": [[0.0, False], [10.0, False], ["nan", True], [11.01, True], [-0.01, True]],
        "message": "particle coordinates are NaN or outside the domain bounds of the cell list",
    }

    # test/gpu.jl:30-36 + docs/literate/src/tut_gpu_usage.jl: 100x100 Float32 lattice,
    # r = 3f0, FullGridCellList over the data extrema, count neighbours (self included).
    cases["gpu_tutorial"] = {
        "source": "test/gpu.jl:35, docs/literate/src/tut_gpu_usage.jl:23-101",
        "n_per_dim": [100, 100], "radius": 3.0, "dtype": "float32",
        "expected_extrema": [11, 29],
    }

    # test/vector_of_vectors.jl:222-227 -- overflowing a column.
    cases["cell_full"] = {
        "source": "test/vector_of_vectors.jl:222-227, src/vector_of_vectors.jl:114-121",
        "message": "cell list is full. Use a larger `max_points_per_cell`.",
    }

    # test/cell_lists/spatial_hashing.jl:2-67 -- hash collisions, with an empty and with a
    # non-empty colliding cell (list_size = n_points), r = 0.1 + 10 eps().
    cases["spatial_hashing_collisions"] = {
        "source": "test/cell_lists/spatial_hashing.jl:2-67",
        "radius": 0.1 + 10 * 2.220446049250313e-16,  # Float64 arithmetic, like Julia's
        "cases": [
            {"coords": [[-0.05, 0.05]], "list_size": 1,
             "colliding_cells": [[-1, 0], [-2, -1]], "cell_points": [1],
             "neighbors": [[1]]},
            {"coords": [[-0.05, 0.05], [-0.15, -0.05]], "list_size": 2,
             "colliding_cells": [[-1, 0], [-2, -1]], "cell_points": [1, 2],
             "neighbors": [[1], [2]]},
        ],
    }

    # test/cell_lists/spatial_hashing.jl:69-121 -- coordinates_flattened.
    cases["coordinates_flattened"] = {
        "source": "test/cell_lists/spatial_hashing.jl:69-121",
        "values": [
            {"cell": [1], "flat": str(1)},
            {"cell": [-1], "flat": str(2**32 - 1)},
            {"cell": [0], "flat": "0"},
            {"cell": [-1, 1], "flat": str(2**32 - 1 + 2**32)},
            {"cell": [1, 0, -1], "flat": str(1 + (2**32 - 1) * 2**64)},
            {"cell": [2**31 - 1], "flat": str(2**31 - 1)},
            {"cell": [-2**31], "flat": str(2**31)},
            {"cell": [-2**31, 2**31 - 1, 0], "flat": str(2**31 + (2**31 - 1) * 2**32)},
        ],
        "inexact": [[2**31], [-2**31 - 1]],
    }

    out = os.path.join(HERE, "reference_known_answers.json")
    with open(out, "w") as f:
        json.dump(cases, f, indent=1)
    print(out)


if __name__ == "__main__":
    main()
