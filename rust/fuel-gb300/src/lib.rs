//! fuel's search and k-means interfaces served by the GB300 engine.
//!
//! * [`GpuLinearScan`] implements fuel's `KnnSearch` and `RangeSearch`
//!   (src/api/search.rs:268-280) for every query type that exposes its
//!   coordinates (`CoordinateSearch`, as fuel's ndarray queries do): kNN
//!   answers are the tie-inclusive lists `KNNHeap::into_vec` returns
//!   (src/api/search.rs:80-151) through `fuelg_knn_ties`, range answers the
//!   sorted lists of `linear_scan_range` (src/api/search.rs:154-166) through
//!   `fuelg_range`.  Distances are bit-identical to fuel's own f32 distances
//!   in the summation order fuel compiles for this host.
//! * [`GpuLinearScan::knn_batch`] / [`GpuLinearScan::precomputed_table`] run
//!   many queries in one call: the batch drivers of python/search.rs:471-514
//!   and the table `PrecomputedKnnSearcher::new` builds
//!   (src/search/precomputed.rs:36-55).
//! * [`GpuLinearScanF64`] does the same for float64 data (fuel's
//!   `build_linear_scan_f64`, python/search.rs:1371-1389) through the exact
//!   FP64 scan (`fuelg_knn_ties_f64`, `fuelg_range_f64`): distances
//!   bit-identical to fuel's own f64 distances.
//! * [`lloyd_gpu`] has the signature of `cluster::kmeans::lloyd`
//!   (src/cluster/kmeans/lloyd.rs:118-125) and runs it through
//!   `fuelg_kmeans_lloyd` with the centres the `Initialization` chooses.
//!
//! Every call is synchronous; calls on one index are serialised inside the
//! library, so the index is `Send + Sync` as fuel's searchers must be.
use std::ptr;

use fuel::api::{CoordinateSearch, DistPair, DistanceSearch, KnnSearch, RangeSearch, VectorData};
use fuel::cluster::kmeans::{Centers, Initialization, KMeansResult};
use fuel_gb300_sys as sys;

/// Distance served on the GPU: fuel's `sqeuclidean` or `euclidean`.
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum Metric {
    SqEuclidean,
    Euclidean,
}

impl Metric {
    /// fuel's metric names (python/mod.rs:42-71) for the two metrics served here.
    pub fn parse(name: &str) -> Option<Metric> {
        match name.to_ascii_lowercase().as_str() {
            "sqeuclidean" | "squared_euclidean" => Some(Metric::SqEuclidean),
            "euclidean" | "l2" => Some(Metric::Euclidean),
            _ => None,
        }
    }
    fn code(self) -> i32 {
        match self {
            Metric::SqEuclidean => sys::FUELG_METRIC_SQEUCLIDEAN,
            Metric::Euclidean => sys::FUELG_METRIC_EUCLIDEAN,
        }
    }
}

/// A linear-scan index resident in GPU memory (the handle owns a device copy).
pub struct GpuLinearScan {
    ix: *mut sys::fuelg_index,
    n: usize,
    d: usize,
    precision: i32,
}

// The library serialises calls on one handle; the handle has no thread affinity.
unsafe impl Send for GpuLinearScan {}
unsafe impl Sync for GpuLinearScan {}

impl Drop for GpuLinearScan {
    fn drop(&mut self) {
        unsafe {
            sys::fuelg_index_destroy(self.ix);
        }
    }
}

/// Tie-inclusive / range lists of a batch, one `Vec<DistPair>` per query row.
fn take_lists(res: *mut sys::fuelg_range_result, m: usize) -> Result<Vec<Vec<DistPair<f32>>>, String> {
    struct Guard(*mut sys::fuelg_range_result);
    impl Drop for Guard {
        fn drop(&mut self) {
            unsafe {
                sys::fuelg_range_free(self.0);
            }
        }
    }
    let _g = Guard(res);
    let (mut mm, mut total) = (0i64, 0i64);
    sys::check(unsafe { sys::fuelg_range_size(res, &mut mm, &mut total) })?;
    let mut off = vec![0i64; m + 1];
    let mut idx = vec![0i64; total.max(1) as usize];
    let mut dist = vec![0f32; total.max(1) as usize];
    sys::check(unsafe { sys::fuelg_range_copy(res, off.as_mut_ptr(), idx.as_mut_ptr(), dist.as_mut_ptr()) })?;
    Ok((0..m)
        .map(|r| {
            (off[r] as usize..off[r + 1] as usize).map(|e| DistPair::new(dist[e], idx[e] as usize)).collect()
        })
        .collect())
}

impl GpuLinearScan {
    /// Upload `n` rows of `d` coordinates (row-major) and build the index.
    /// `precision`: one of `sys::FUELG_PREC_*` (`FUELG_PREC_AUTO` lets the
    /// engine pick; every tier returns the same bits).
    pub fn new(data: &[f32], n: usize, d: usize, metric: Metric, precision: i32) -> Result<Self, String> {
        if data.len() != n * d {
            return Err(format!("data holds {} values, expected n*d = {}", data.len(), n * d));
        }
        let mut ix = ptr::null_mut();
        sys::check(unsafe {
            sys::fuelg_index_create(data.as_ptr(), n as i64, d as i32, metric.code(), sys::FUELG_ORDER_HOST, &mut ix)
        })?;
        Ok(GpuLinearScan { ix, n, d, precision })
    }

    /// Index every row of a fuel data set.
    pub fn from_data<A: VectorData<f32>>(data: &A, metric: Metric, precision: i32) -> Result<Self, String> {
        let (n, d) = (data.nrows(), data.ncols());
        let mut rows = Vec::with_capacity(n * d);
        for i in 0..n {
            rows.extend_from_slice(data.point(i));
        }
        Self::new(&rows, n, d, metric, precision)
    }

    pub fn len(&self) -> usize { self.n }
    pub fn is_empty(&self) -> bool { self.n == 0 }
    pub fn dims(&self) -> usize { self.d }

    /// Tie-inclusive kNN lists of `m` query rows (row-major, `m * d` values).
    /// `exclude_mode`: `FUELG_EXCLUDE_NONE`, `_LINEAR` (search k, drop index i
    /// from row i: python/search.rs:485-488) or `_KPLUS1` (search k+1, drop
    /// self: python/search.rs:1163-1170).
    pub fn knn_batch(&self, queries: &[f32], k: usize, exclude_mode: i32) -> Result<Vec<Vec<DistPair<f32>>>, String> {
        let m = queries.len() / self.d.max(1);
        let mut res = ptr::null_mut();
        sys::check(unsafe {
            sys::fuelg_knn_ties(self.ix, queries.as_ptr(), m as i64, k as i32, exclude_mode, self.precision, &mut res,
                                ptr::null_mut())
        })?;
        take_lists(res, m)
    }

    /// The kNN table of every indexed point to `max_k` neighbours with ties
    /// (self included, at distance 0): what `PrecomputedKnnSearcher::new`
    /// stores, computed as one self-join on the device with no query upload.
    pub fn precomputed_table(&self, max_k: usize) -> Result<Vec<Vec<DistPair<f32>>>, String> {
        let max_k = max_k.min(self.n);
        let mut res = ptr::null_mut();
        sys::check(unsafe {
            sys::fuelg_knn_ties(self.ix, ptr::null(), self.n as i64, max_k as i32, sys::FUELG_EXCLUDE_NONE,
                                self.precision, &mut res, ptr::null_mut())
        })?;
        take_lists(res, self.n)
    }

    /// Sorted range lists of `m` query rows (radius cast to f32 as
    /// python/search.rs:781-783 does).
    pub fn range_batch(&self, queries: &[f32], radius: f32, exclude_self: bool)
        -> Result<Vec<Vec<DistPair<f32>>>, String> {
        let m = queries.len() / self.d.max(1);
        let mut res = ptr::null_mut();
        sys::check(unsafe {
            sys::fuelg_range(self.ix, queries.as_ptr(), m as i64, radius as f64, exclude_self as i32, &mut res,
                             ptr::null_mut())
        })?;
        take_lists(res, m)
    }

    fn coords<Q: CoordinateSearch<f32, f32> + ?Sized>(&self, q: &Q) -> Vec<f32> {
        (0..self.d).map(|axis| q.query_coordinate(axis)).collect()
    }
}

impl<Q> KnnSearch<f32, Q> for GpuLinearScan
where
    Q: DistanceSearch<f32> + CoordinateSearch<f32, f32> + ?Sized,
{
    /// `linear_scan_knn` (src/api/search.rs:169-184): the k nearest plus every
    /// tie at the k-th distance, sorted by (distance, index).
    fn search_knn(&self, query: &Q, k: usize) -> Vec<DistPair<f32>> {
        if k == 0 || self.n == 0 {
            return Vec::new();
        }
        let q = self.coords(query);
        self.knn_batch(&q, k, sys::FUELG_EXCLUDE_NONE)
            .map(|mut rows| rows.pop().unwrap_or_default())
            .unwrap_or_else(|e| panic!("GPU kNN failed: {e}"))
    }
}

impl<Q> RangeSearch<f32, Q> for GpuLinearScan
where
    Q: DistanceSearch<f32> + CoordinateSearch<f32, f32> + ?Sized,
{
    /// `linear_scan_range` (src/api/search.rs:154-166).
    fn search_range(&self, query: &Q, radius: f32) -> Vec<DistPair<f32>> {
        if self.n == 0 {
            return Vec::new();
        }
        let q = self.coords(query);
        self.range_batch(&q, radius, false)
            .map(|mut rows| rows.pop().unwrap_or_default())
            .unwrap_or_else(|e| panic!("GPU range search failed: {e}"))
    }
}

/// Tie-inclusive / range lists of a float64 batch, one `Vec<DistPair>` per query row.
fn take_lists_f64(res: *mut sys::fuelg_range_result, m: usize) -> Result<Vec<Vec<DistPair<f64>>>, String> {
    struct Guard(*mut sys::fuelg_range_result);
    impl Drop for Guard {
        fn drop(&mut self) {
            unsafe {
                sys::fuelg_range_free(self.0);
            }
        }
    }
    let _g = Guard(res);
    let (mut mm, mut total) = (0i64, 0i64);
    sys::check(unsafe { sys::fuelg_range_size(res, &mut mm, &mut total) })?;
    let mut off = vec![0i64; m + 1];
    let mut idx = vec![0i64; total.max(1) as usize];
    let mut dist = vec![0f64; total.max(1) as usize];
    sys::check(unsafe { sys::fuelg_range_copy_f64(res, off.as_mut_ptr(), idx.as_mut_ptr(), dist.as_mut_ptr()) })?;
    Ok((0..m)
        .map(|r| {
            (off[r] as usize..off[r + 1] as usize).map(|e| DistPair::new(dist[e], idx[e] as usize)).collect()
        })
        .collect())
}

/// A float64 linear-scan index resident in GPU memory: fuel's
/// `build_linear_scan_f64` (python/search.rs:1371-1389) on the exact FP64 scan.
pub struct GpuLinearScanF64 {
    ix: *mut sys::fuelg_index,
    n: usize,
    d: usize,
}

unsafe impl Send for GpuLinearScanF64 {}
unsafe impl Sync for GpuLinearScanF64 {}

impl Drop for GpuLinearScanF64 {
    fn drop(&mut self) {
        unsafe {
            sys::fuelg_index_destroy(self.ix);
        }
    }
}

impl GpuLinearScanF64 {
    /// Upload `n` rows of `d` coordinates (row-major) and build the index.
    pub fn new(data: &[f64], n: usize, d: usize, metric: Metric) -> Result<Self, String> {
        if data.len() != n * d {
            return Err(format!("data holds {} values, expected n*d = {}", data.len(), n * d));
        }
        let mut ix = ptr::null_mut();
        sys::check(unsafe {
            sys::fuelg_index_create_f64(data.as_ptr(), n as i64, d as i32, metric.code(), sys::FUELG_ORDER_HOST,
                                        &mut ix)
        })?;
        Ok(GpuLinearScanF64 { ix, n, d })
    }

    /// Index every row of a fuel data set.
    pub fn from_data<A: VectorData<f64>>(data: &A, metric: Metric) -> Result<Self, String> {
        let (n, d) = (data.nrows(), data.ncols());
        let mut rows = Vec::with_capacity(n * d);
        for i in 0..n {
            rows.extend_from_slice(data.point(i));
        }
        Self::new(&rows, n, d, metric)
    }

    pub fn len(&self) -> usize { self.n }
    pub fn is_empty(&self) -> bool { self.n == 0 }
    pub fn dims(&self) -> usize { self.d }

    /// Tie-inclusive kNN lists of `m` query rows, exclude rules as
    /// [`GpuLinearScan::knn_batch`].
    pub fn knn_batch(&self, queries: &[f64], k: usize, exclude_mode: i32) -> Result<Vec<Vec<DistPair<f64>>>, String> {
        let m = queries.len() / self.d.max(1);
        let mut res = ptr::null_mut();
        sys::check(unsafe {
            sys::fuelg_knn_ties_f64(self.ix, queries.as_ptr(), m as i64, k as i32, exclude_mode, &mut res,
                                    ptr::null_mut())
        })?;
        take_lists_f64(res, m)
    }

    /// The kNN table of every indexed point to `max_k` neighbours with ties.
    pub fn precomputed_table(&self, max_k: usize) -> Result<Vec<Vec<DistPair<f64>>>, String> {
        let max_k = max_k.min(self.n);
        let mut res = ptr::null_mut();
        sys::check(unsafe {
            sys::fuelg_knn_ties_f64(self.ix, ptr::null(), self.n as i64, max_k as i32, sys::FUELG_EXCLUDE_NONE,
                                    &mut res, ptr::null_mut())
        })?;
        take_lists_f64(res, self.n)
    }

    /// Sorted range lists of `m` query rows (f64 radius).
    pub fn range_batch(&self, queries: &[f64], radius: f64, exclude_self: bool)
        -> Result<Vec<Vec<DistPair<f64>>>, String> {
        let m = queries.len() / self.d.max(1);
        let mut res = ptr::null_mut();
        sys::check(unsafe {
            sys::fuelg_range_f64(self.ix, queries.as_ptr(), m as i64, radius, exclude_self as i32, &mut res,
                                 ptr::null_mut())
        })?;
        take_lists_f64(res, m)
    }

    fn coords<Q: CoordinateSearch<f64, f64> + ?Sized>(&self, q: &Q) -> Vec<f64> {
        (0..self.d).map(|axis| q.query_coordinate(axis)).collect()
    }
}

impl<Q> KnnSearch<f64, Q> for GpuLinearScanF64
where
    Q: DistanceSearch<f64> + CoordinateSearch<f64, f64> + ?Sized,
{
    /// `linear_scan_knn` on f64 data: the k nearest plus every tie at the k-th
    /// distance, sorted by (distance, index).
    fn search_knn(&self, query: &Q, k: usize) -> Vec<DistPair<f64>> {
        if k == 0 || self.n == 0 {
            return Vec::new();
        }
        let q = self.coords(query);
        self.knn_batch(&q, k, sys::FUELG_EXCLUDE_NONE)
            .map(|mut rows| rows.pop().unwrap_or_default())
            .unwrap_or_else(|e| panic!("GPU kNN failed: {e}"))
    }
}

impl<Q> RangeSearch<f64, Q> for GpuLinearScanF64
where
    Q: DistanceSearch<f64> + CoordinateSearch<f64, f64> + ?Sized,
{
    /// `linear_scan_range` on f64 data.
    fn search_range(&self, query: &Q, radius: f64) -> Vec<DistPair<f64>> {
        if self.n == 0 {
            return Vec::new();
        }
        let q = self.coords(query);
        self.range_batch(&q, radius, false)
            .map(|mut rows| rows.pop().unwrap_or_default())
            .unwrap_or_else(|e| panic!("GPU range search failed: {e}"))
    }
}

/// `cluster::kmeans::lloyd` (src/cluster/kmeans/lloyd.rs:118-125) on the GPU:
/// the `Initialization` picks the starting centres on the host, then
/// `fuelg_kmeans_lloyd` runs the loop (initial assignment in the
/// `vec_pairwise_sqdist` order, later passes in the `math::sqdist` order,
/// first index wins, `changed == 0` stop, the tol rule of lloyd.rs:147-153).
/// Centres are the correctly rounded means of exact sums (fuel's f32 running
/// sums depend on the rayon thread count); assignments given the same centres
/// are bit-identical to fuel's.  The inertia is the FP64 sum of the final
/// pass, returned as f32.
pub fn lloyd_gpu<I, A>(data: &A, k: usize, init: &mut I, maxiter: usize, tol: f32) -> Result<KMeansResult<f32>, String>
where
    I: Initialization<f32>,
    A: VectorData<f32> + Sync,
{
    let (n, d) = (data.nrows(), data.ncols());
    if k == 0 || n == 0 {
        return Err(format!("k-means needs k > 0 and n > 0 (k={k}, n={n})"));
    }
    let mut cent = Centers::<f32>::new(k, d);
    init.init(data, &mut cent, k);
    let c0 = cent.into_ndarray();
    let c0 = c0.as_slice().ok_or("centres are not contiguous")?;
    let mut rows = Vec::with_capacity(n * d);
    for i in 0..n {
        rows.extend_from_slice(data.point(i));
    }
    let mut centers = vec![0f32; k * d];
    let mut labels = vec![0i64; n];
    let (mut iters, mut inertia) = (0i32, 0f64);
    sys::check(unsafe {
        sys::fuelg_kmeans_lloyd(rows.as_ptr(), n as i64, d as i32, k as i32, c0.as_ptr(), maxiter.max(1) as i32,
                                tol as f64, sys::FUELG_PREC_AUTO, sys::FUELG_ORDER_HOST, 0, centers.as_mut_ptr(),
                                labels.as_mut_ptr(), &mut iters, &mut inertia, ptr::null_mut())
    })?;
    let centers = ndarray::Array2::from_shape_vec((k, d), centers).map_err(|e| e.to_string())?;
    Ok(KMeansResult::with_inertia(centers, labels.into_iter().map(|v| v as usize).collect(), iters as usize,
                                  inertia as f32))
}

/// Cooperative cancellation: fuel's signal poll (src/api/parallel.rs:145-173)
/// calls this when SHUTDOWN_REQUESTED is set; the running call then returns
/// FUELG_ECANCELLED, which maps to fuel's `Err("interrupted")`.
pub fn cancel_running_calls() {
    unsafe {
        sys::fuelg_cancel();
    }
}
